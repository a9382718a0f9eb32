// fst_batch_w64.cu — the persistent batched RHS kernels of tile width 64
// (every tile height and species count; see fst_batch_dev.cuh).
#include "fst_batch_dev.cuh"

namespace fstb {
const void* brhs_kernel_w64(int tyy, int nv) { return brhs_kernel_for<64>(tyy, nv); }
}  // namespace fstb
