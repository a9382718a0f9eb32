// fst_hybrid.cu — learned smoothness classifier (FST_MODE_HYBRID).
#include "fst_internal.h"
int fst_hybrid_alloc(const fst_config&, const Geo&, MixedBufs& b, const fst_alloc_fn&) {
  b.hyb_active = false;
  return FST_OK;
}
int fst_hybrid_classify(const Geo&, const Phys&, const MixedBufs&, const MixedView&, cudaStream_t,
                        Prof*, const unsigned char** smooth) {
  *smooth = nullptr;
  return 0;
}
