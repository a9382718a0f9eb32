// fst_batch_dev.cuh — device side of the batched 2D ensemble shared by
// fst_batch.cu (orchestration, ghost fills, primitive pass, autotuner) and
// the three units that instantiate the persistent RHS kernel per tile width
// (fst_batch_w16.cu, fst_batch_w32.cu, fst_batch_w64.cu; split so that the
// 48 instantiations compile in parallel).
#pragma once

#include "fst_mixed_dev.cuh"

namespace fstb {

using namespace fstm;

struct BCase {
  Geo g;
  MixedView M;
  double *Ua, *Ub;
  unsigned long long* red;  // 2 keys
  float* Q;                 // writable views of the mixed buffers
  float *rho32, *vel32, *T32, *nrg, *C, *lo;
  double *p64, *rho64;
  int bc[4];     // xmin, xmax, ymin, ymax
  int per[2];    // x, y periodic
};

__device__ __forceinline__ int find_case(const int* __restrict__ off, int n, int x) {
  // largest c with off[c] <= x (off has n+1 entries, off[0] = 0)
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

// persistent RHS + RK stage over the (case, tile) work list: block b takes
// work items b, b + gridDim.x, ...; item w is tile w - tile_off[c] of case c
// (tiles of a case in row-major order, (nci + TXX - 2) / (TXX - 1) per row).
template <int NV, int TYY, int TXX>
__global__ void __launch_bounds__(TXX * TYY) k_brhs(const BCase* __restrict__ cs,
                                                    const Phys* __restrict__ Ps,
                                                    const int* __restrict__ tile_off, int ncase,
                                                    int stage) {
  __shared__ float sG[TYY][TXX][NV];
  __shared__ float sE[TYY * (TXX > 32 ? TXX / 32 : 1)][NV];
  const int ntile = tile_off[ncase];
  for (int w = blockIdx.x; w < ntile; w += gridDim.x) {
    const int c = find_case(tile_off, ncase, w);
    const BCase& B = cs[c];
    const Phys& P = Ps[c];
    const int ntx = (B.g.nci + TXX - 2) / (TXX - 1);
    const int local = w - tile_off[c];
    // stage 1: Ub = Ua + hdt*R(Ua); stage 2: Ua = Ua + dt*R(Ub)
    rhs2d_tile<NV, false, TYY, TXX>(B.g, P, B.M, B.red, nullptr, B.Ua, stage == 1 ? B.Ub : B.Ua,
                                    stage == 1 ? P.hdt : P.dt, nullptr, local % ntx, local / ntx,
                                    sG, sE);
    __syncthreads();
  }
}

// the k_brhs instantiation for (TXX, TYY, nv); nullptr for a shape that is
// not instantiated.  nv above 8 takes the NVMAX kernel.
template <int TXX>
const void* brhs_kernel_for(int tyy, int nv) {
  auto pick = [nv](auto k4, auto k5, auto k6, auto k7, auto k8, auto kmax) -> const void* {
    switch (nv) {
      case 4: return (const void*)k4;
      case 5: return (const void*)k5;
      case 6: return (const void*)k6;
      case 7: return (const void*)k7;
      case 8: return (const void*)k8;
      default: return (const void*)kmax;
    }
  };
#define FST_BRHS_SET(H)                                                                       \
  pick(k_brhs<4, H, TXX>, k_brhs<5, H, TXX>, k_brhs<6, H, TXX>, k_brhs<7, H, TXX>,            \
       k_brhs<8, H, TXX>, k_brhs<NVMAX, H, TXX>)
  if (tyy == 4) return FST_BRHS_SET(4);
  if (tyy == 8) return FST_BRHS_SET(8);
  if constexpr (TXX * 16 <= 512) {
    if (tyy == 16) return FST_BRHS_SET(16);
  }
#undef FST_BRHS_SET
  return nullptr;
}

// defined in fst_batch_w16.cu / fst_batch_w32.cu / fst_batch_w64.cu
const void* brhs_kernel_w16(int tyy, int nv);
const void* brhs_kernel_w32(int tyy, int nv);
const void* brhs_kernel_w64(int tyy, int nv);

}  // namespace fstb
