// fst_mixed.cu — placeholder until the mixed-precision path lands.
#include "fst_internal.h"
size_t fst_mixed_work_doubles_per_cell(const fst_config&, const Geo&) { return 0; }
int fst_mixed_alloc(const fst_config&, const Geo&, MixedBufs&, const fst_alloc_fn&) {
  return FST_ERR_UNSUPPORTED;
}
int fst_mixed_stage(const Geo&, const Phys&, const fst_config&, const MixedBufs&, const double*,
                    const double*, double*, double, double*, bool, cudaStream_t, Prof*) {
  return 0;
}
int fst_mixed_secondary(const Geo&, const Phys&, const MixedBufs&, const double*, cudaStream_t,
                        const double**, const double**, const double**, const double**) {
  return 0;
}
double fst_mixed_flagged_fraction(const MixedBufs&, cudaStream_t) { return 0.0; }
