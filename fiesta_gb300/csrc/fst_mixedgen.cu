// fst_mixedgen.cu — the mixed-precision form of gen3d_func::compute
// (src/gen3d.cpp:338-370) on generalized (curvilinear) grids.
//
// The face kernels of the 3D mixed path (species and momentum/energy WENO5)
// run unchanged on the contravariant velocity; what is specific to the
// generalized module is here:
//   k_metric_pair   the FP64 metric tensor as FP32 pairs hi + lo (once, at
//                   fst_set_grid), in the primitives' padded layout
//   k_gen_tvel      the contravariant velocity u^a = sum_b m(a,b) u_b from the
//                   primitive pass's velocity, in place (computeGenVelocity3D,
//                   src/velocity.hpp:23-48)
//   k_gen_cell      applyGenPressureGradient3D (src/presgrad.hpp:72-146):
//                   R_w = -sum_a D_a(p m(a,w)) with the fourth-order difference
//                   D, then U_new = U_old + coef R for the momenta; energy and
//                   C-variables (no cell term) get U_old + coef*0
// Precision of the pressure term: p (hi + lo pair of the primitive pass)
// times m (hi + lo) is formed as an FP32 pair (the rounding error of ph*mh
// recovered by an FMA), and the differences of neighbouring products are
// taken hi with hi (exact for close values) and lo with lo, so only the final
// combination rounds (relative error ~1e-7 of the term), as the cartesian
// mixed path does for its pressure gradient.
//
// Built without fast math: the pair arithmetic relies on IEEE products and
// fused multiply-adds, written with explicit intrinsics.
#include "fst_internal.h"

namespace {

inline unsigned cdiv(long long a, int b) { return (unsigned)((a + b - 1) / b); }

// Both per-cell kernels below run one block per grid row (j, k), ghosts
// included, threads along i.

// metric (a, b) of a cell as FP32 hi [9 fields] and lo [9 fields]
__global__ void __launch_bounds__(128) k_metric_pair(Geo g, Geo gq, const double* __restrict__ met,
                                                     float* __restrict__ metf) {
  const int j = (int)(blockIdx.x % g.ngj), k = (int)(blockIdx.x / g.ngj);
  for (int i = threadIdx.x; i < g.ngi; i += 128) {
    const long long c = (long long)i + g.sy * j + g.sz * k;
    const long long q = (long long)i + gq.sy * j + gq.sz * k;
#pragma unroll
    for (int n = 0; n < 9; ++n) {
      const double m = met[c + g.sv * n];
      const float h = __double2float_rn(m);
      metf[q + gq.sv * n] = h;
      metf[q + gq.sv * (9 + n)] = __double2float_rn(m - (double)h);
    }
  }
}

// contravariant velocity over every cell (ghosts included: the face
// kernels' stencils read them), in place
__global__ void __launch_bounds__(128) k_gen_tvel(Geo gq, int ngi, int ngj,
                                                  const float* __restrict__ metf,
                                                  float* __restrict__ vel) {
  const int j = (int)(blockIdx.x % ngj), k = (int)(blockIdx.x / ngj);
  const long long sv = gq.sv;
  for (int i = threadIdx.x; i < ngi; i += 128) {
    const long long q = (long long)i + gq.sy * j + gq.sz * k;
    const float u0 = vel[q], u1 = vel[q + sv], u2 = vel[q + 2 * sv];
    float t[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)  // m(a, b) at field a + 3b
      t[a] = __fmaf_rn(metf[q + sv * (a + 6)], u2,
                       __fmaf_rn(metf[q + sv * (a + 3)], u1, __fmul_rn(metf[q + sv * a], u0)));
#pragma unroll
    for (int a = 0; a < 3; ++a) vel[q + sv * a] = t[a];
  }
}

// p*m at one stencil point as an FP32 pair (hi exact product rounding, lo the
// rest): (ph + pl)(mh + ml) ~ ph*mh + [err(ph*mh) + ph*ml + pl*mh]
struct Pair {
  float h, l;
};
__device__ __forceinline__ Pair pm(float ph, float pl, float mh, float ml) {
  const float h = __fmul_rn(ph, mh);
  const float e = __fmaf_rn(ph, mh, -h);
  return {h, __fmaf_rn(pl, mh, __fmaf_rn(ph, ml, e))};
}

// thread per interior cell
__global__ void __launch_bounds__(256) k_gen_cell(Geo g, Geo gq, MixedView M,
                                                  const float* __restrict__ metf,
                                                  const double* __restrict__ Uold,
                                                  double* __restrict__ Unew, double coef,
                                                  double* __restrict__ Rout) {
  const int i = g.ng + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int j = g.ng + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int k = g.ng + (int)blockIdx.z;
  if (i >= g.ngi - g.ng || j >= g.ngj - g.ng) return;
  const long long q = (long long)i + gq.sy * j + gq.sz * k;
  const long long c = (long long)i + g.sy * j + g.sz * k;
  const long long st[3] = {1, gq.sy, gq.sz};
  const long long sv = gq.sv;
  const float* ph = M.pp;
  const float* pl = M.pp + sv;
  float s[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const long long o = st[a];
    const long long pts[4] = {q - 2 * o, q - o, q + o, q + 2 * o};
    Pair t[4][3];  // p*m(a, w) at the four points, each pressure read once
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      const long long x = pts[n];
      const float h = ph[x], l = pl[x];
#pragma unroll
      for (int w = 0; w < 3; ++w) {
        const float* mf = metf + sv * (a + 3 * w);
        t[n][w] = pm(h, l, mf[x], mf[x + 9 * sv]);
      }
    }
    // (t(-2) - 8 t(-1) + 8 t(+1) - t(+2)) / 12 with close values differenced first
#pragma unroll
    for (int w = 0; w < 3; ++w) {
      const float A = __fadd_rn(__fsub_rn(t[2][w].h, t[1][w].h), __fsub_rn(t[2][w].l, t[1][w].l));
      const float B = __fadd_rn(__fsub_rn(t[3][w].h, t[0][w].h), __fsub_rn(t[3][w].l, t[0][w].l));
      s[w] = __fadd_rn(s[w], __fmul_rn(__fmaf_rn(8.0f, A, -B), 1.0f / 12.0f));
    }
  }
#pragma unroll
  for (int w = 0; w < 3; ++w) {
    const double r = (double)(-s[w]);
    const long long a = c + g.sv * w;
    if (Rout) Rout[a] = r;
    else Unew[a] = Uold[a] + coef * r;
  }
  // energy and the C-equation variables: no cell term; the face kernel adds
  // the energy's fluxes to this
  for (int v = 3; v < g.nvt; ++v) {
    if (v >= 4 && v < g.nv) continue;  // species: k_mspec3d
    const long long a = c + g.sv * v;
    if (Rout) Rout[a] = 0.0;
    else Unew[a] = Uold[a] + coef * 0.0;
  }
}

}  // namespace

int fst_mixedgen_pair(const Geo& g, const Geo& gq, const double* met, float* metf,
                      cudaStream_t st) {
  k_metric_pair<<<(unsigned)g.ngj * g.ngk, 128, 0, st>>>(g, gq, met, metf);
  return 1;
}

int fst_mixedgen_tvel(const Geo& g, const Geo& gq, const float* metf, float* vel,
                      cudaStream_t st) {
  k_gen_tvel<<<(unsigned)g.ngj * g.ngk, 128, 0, st>>>(gq, g.ngi, g.ngj, metf, vel);
  return 1;
}

int fst_mixedgen_cell(const Geo& g, const Geo& gq, const MixedView& M, const float* metf,
                      const double* Uold, double* Unew, double coef, double* Rout,
                      cudaStream_t st) {
  const dim3 blk(32, 8, 1), grd(cdiv(g.nci, 32), cdiv(g.ncj, 8), g.nck);
  k_gen_cell<<<grd, blk, 0, st>>>(g, gq, M, metf, Uold, Unew, coef, Rout);
  return 1;
}
