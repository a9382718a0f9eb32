// fst_batch_w16.cu — the persistent batched RHS kernels of tile width 16
// (every tile height and species count; see fst_batch_dev.cuh).
#include "fst_batch_dev.cuh"

namespace fstb {
const void* brhs_kernel_w16(int tyy, int nv) { return brhs_kernel_for<16>(tyy, nv); }
}  // namespace fstb
