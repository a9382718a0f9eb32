// fst_common.cuh — shared device-side definitions of libfst.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/fst.h"

#define FST_MAXV (4 + FST_MAX_SPECIES + 5)

// Grid geometry and strides of one field in HBM.  Fields are stored like the
// reference's CUDA build, LayoutLeft with i fastest:
//   a[i + sy*j + sz*k + sv*v],  sy = ngi, sz = ngi*ngj, sv = ngi*ngj*ngk.
struct Geo {
  int ndim, ng, nci, ncj, nck, ngi, ngj, ngk;
  int ns, nv, nvt;
  long long sy, sz, sv;
};

// Division by a run-time constant d.  When d is a power of two, a/d equals
// a*(1/d) exactly for every a (both are the correctly rounded a*2^-k), so the
// multiply is used; otherwise the IEEE division.  Results are bit-identical
// to a/d either way.
struct DivC {
  double d, inv;  // inv = 1/d if d is a power of two, else 0
  __device__ __forceinline__ double operator()(double a) const {
    return inv != 0.0 ? a * inv : a / d;
  }
};

// Physics constants of one run, passed by value to the kernels.
struct Phys {
  int ns, nv, nvt, visc, ceq, buoyancy;
  int scheme;  // 2D flux: 1 WENO5, 2 centered4, 3 QUICK (src/cart2d.cpp:165-172)
  // species constants of calculateRhoPT (src/secondary.hpp:127-135):
  //   cp_s = gammas*Rs/(gammas-1), cv_s = Rs/(gammas-1), Rs = cd(7+3s)
  double cp_s[FST_MAX_SPECIES], cv_s[FST_MAX_SPECIES], mu_s[FST_MAX_SPECIES];
  double rm_s[FST_MAX_SPECIES];  // cp_s - cv_s = Rs (mixed path)
  // the same with the stride-2 species table read by maxWaveSpeed2D
  // (src/ceq.hpp:61-66): gammas = cd(6+2s), Rs = cd(7+2s)
  double cp2_s[FST_MAX_SPECIES], cv2_s[FST_MAX_SPECIES];
  double dx, dy, dz;
  DivC ddx, ddy, ddz;     // x/dx, x/dy, x/dz
  DivC d4x, d4y, d4z;     // x/(4*dx) ... (viscous and C-equation tangential terms)
  double d12x, d12y, d12z;  // 12.0*dx, 12.0*dy, 12.0*dz (4th-order derivatives)
  double d12pz;           // 12.0*cd(2): the reference's dz = cd(2) in presgrad3D
  double r12x, r12y, r12pz;  // their reciprocals (mixed path)
  double dt, hdt;         // dt and 0.5f*dt
  double kap, eps, alpha, g, rho_ref;
  double dxmag2;          // dx^2+dy^2(+dz^2): alpha numerator
  double dxmag;           // sqrt(dx^2+dy^2(+dz^2)): updateCeq cell size
  double mu2d;            // constant 2D viscosity 2.928e-5 (src/viscosity.hpp:62-63)
  double kheat2d;         // 2D heat conductivity 0.026 (src/viscosity.hpp:117)
  // FP32 copies for the mixed path: cv_s, R_s = cp_s - cv_s, mu_s, and the
  // stride-2 table constants
  float cv_f[FST_MAX_SPECIES], rm_f[FST_MAX_SPECIES], mu_f[FST_MAX_SPECIES];
  // low parts of cv_s and R_s as FP32 pairs (cv_f + cv_lf, rm_f + rm_lf)
  float cv_lf[FST_MAX_SPECIES], rm_lf[FST_MAX_SPECIES];
  float cv2_f[FST_MAX_SPECIES], cp2_f[FST_MAX_SPECIES];
  // FP32 copies of the grid constants (mixed path)
  float rd_f[3];    // 1/dx, 1/dy, 1/dz
  float r12_f[3];   // 1/(12 dx), 1/(12 dy), 1/(12 dz)
  float dxmag_f, dxmag2_f, eps_f, kap_f, alpha_f, mu2d_f, kheat_f;
};

// The bit pattern of x through an opaque register move.  Integer tests on
// the bits then stay integer tests: an optimiser may otherwise rewrite a
// masked compare such as (bits & 0x7FF..F) >= c as an ordered FP compare
// |x| >= c', which is false for NaN where the integer test is true.
__device__ __forceinline__ unsigned long long fst_bits(double x) {
  unsigned long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
}

// --- order-preserving encoding of doubles for atomicMax -------------------
__device__ __forceinline__ unsigned long long fst_key(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double fst_unkey(unsigned long long k) {
  unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, 8);
  return d;
#endif
}
// Kokkos::Max starts from -DBL_MAX and `if (s > lmax)` never takes a NaN.
#define FST_KEY_LOWEST 0x0010000000000000ull /* fst_key(-DBL_MAX) */

// Warp-wide max of per-thread maxima that already skipped NaN.
__device__ __forceinline__ double fst_warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w > v) ? w : v;  // NaN never wins, as in the reference reducer
  }
  return v;
}

// finiteness from the exponent bits (integer ops, not the FP64 pipe)
__device__ __forceinline__ bool fst_finite(double x) {
  return (fst_bits(x) & 0x7FF0000000000000ull) != 0x7FF0000000000000ull;
}

// Linear index helpers
__device__ __forceinline__ long long fst_idx(const Geo& g, int i, int j, int k) {
  return (long long)i + g.sy * j + g.sz * k;
}

// The ghost cells of a grid in a flat order: the ghost planes in k (3D), the
// ghost rows in j of the interior planes, the ghost columns in i of the
// interior rows (each part contiguous along i).  fst_shell_count gives their
// number; fst_shell_cell maps t in [0, count) to (i, j, k).
__host__ __device__ __forceinline__ long long fst_shell_count(const Geo& g) {
  const int ngz = g.ndim == 3 ? g.ng : 0;
  const long long nk = g.ngk - 2 * ngz, nj = g.ngj - 2 * g.ng;
  return 2LL * ngz * g.ngi * g.ngj + nk * 2 * g.ng * g.ngi + nk * nj * 2 * g.ng;
}
__device__ __forceinline__ void fst_shell_cell(const Geo& g, long long t, int& i, int& j,
                                               int& k) {
  const int ng = g.ng, ngz = g.ndim == 3 ? g.ng : 0;
  const int nj = g.ngj - 2 * ng, nk = g.ngk - 2 * ngz;
  const long long pl = (long long)g.ngi * g.ngj;
  const long long nA = 2LL * ngz * pl, nB = (long long)nk * 2 * ng * g.ngi;
  if (t < nA) {
    const long long p = t / pl, r = t - p * pl;
    k = p < ngz ? (int)p : g.ngk - 2 * ngz + (int)p;
    j = (int)(r / g.ngi);
    i = (int)(r - (long long)j * g.ngi);
  } else if (t < nA + nB) {
    const long long u = t - nA, row = u / g.ngi;
    i = (int)(u - row * g.ngi);
    const int kk = (int)(row / (2 * ng)), jj = (int)(row - (long long)kk * 2 * ng);
    k = ngz + kk;
    j = jj < ng ? jj : g.ngj - 2 * ng + jj;
  } else {
    const long long u = t - nA - nB, row = u / (2 * ng);
    const int ii = (int)(u - row * 2 * ng);
    const int kk = (int)(row / nj), jj = (int)(row - (long long)kk * nj);
    k = ngz + kk;
    j = ng + jj;
    i = ii < ng ? ii : g.ngi - 2 * ng + ii;
  }
}
