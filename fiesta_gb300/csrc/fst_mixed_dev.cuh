// fst_mixed_dev.cuh — device code of the mixed-precision path, shared by the
// single-case kernels (fst_mixed.cu) and the batched 2D ensemble
// (fst_batch.cu).  See fst_mixed.cu for the design.
#pragma once
#include "fst_internal.h"

namespace fstm {

constexpr int TX = 32;  // tile width (threads along i)
constexpr int TY = 8;   // tile height (threads along j)
constexpr int KZ = 16;  // planes per block along k
constexpr int NVMAX = 4 + FST_MAX_SPECIES;

// ---------------------------------------------------------------------------
// primitives
// ---------------------------------------------------------------------------
// FP64 <-> FP32 conversions on the integer pipe.  GB300's FP64 unit also
// executes the F2F conversions, at the FP64 rate; these rebias the exponent
// and round the mantissa with integer operations instead.  Values outside
// the FP32 normal range go to signed zero / infinity (no FP32 denormals);
// NaN stays NaN; mantissa ties round away from zero.
__device__ __forceinline__ float d2f(double x) {
  const unsigned int hi = (unsigned int)__double2hiint(x), lo = (unsigned int)__double2loint(x);
  // the low 9 exponent bits and 23 mantissa bits in one funnel shift, then
  // the exponent rebiased 1023 -> 127 (exact modulo 2^32 for the normal
  // range) and the dropped bits rounded
  unsigned int bits = __funnelshift_l(lo, hi, 3) - (896u << 23);
  bits += (lo >> 28) & 1u;  // a carry rounds into the exponent
  // outside the FP32 normal range (selects, no branch: zeros are common)
  const unsigned int ex = (hi >> 20) & 0x7FFu;
  const unsigned int big = (ex == 0x7FFu && ((hi & 0xFFFFFu) | lo)) ? 0x7FC00000u : 0x7F800000u;
  bits = ex < 897u ? 0u : bits;
  bits = ex > 1150u ? big : bits;
  return __uint_as_float((hi & 0x80000000u) | bits);
}
__device__ __forceinline__ double f2d(float x) {
  const unsigned int f = __float_as_uint(x), a = f & 0x7FFFFFFFu;
  unsigned int hi = (a >> 3) + (896u << 20), lo = f << 29;  // exponent rebiased 127 -> 1023
  // zero / FP32 denormal, inf / NaN (selects, no branch)
  const unsigned int m = a & 0x7FFFFFu;
  const unsigned int special = 0x7FF00000u | (m >> 3) | (m ? 0x80000u : 0u);
  hi = a >= 0x7F800000u ? special : hi;
  hi = a < 0x00800000u ? 0u : hi;
  lo = a < 0x00800000u ? 0u : lo;
  return __hiloint2double((int)(hi | (f & 0x80000000u)), (int)lo);
}

// FP64 reciprocal by one Newton-Raphson step from the correctly rounded FP32
// reciprocal: relative error below ~1e-14 (the square of the seed's 2^-24),
// for arguments inside the FP32 range, which holds for the densities and heat
// capacities it is used on.
__device__ __forceinline__ double rcp64(double x) {
  const double r = f2d(__frcp_rn(d2f(x)));
  return fma(r, fma(-x, r, 1.0), r);
}

// ---------------------------------------------------------------------------
// FP32 pairs ("double-float"): a value carried as h + l with |l| at most
// about ulp(h), ~48 significant bits.  GB300 retires FP64 instructions at
// 1/64 of the FP32 rate, so quantities that need more than FP32 accuracy are
// formed with error-free transformations on the FP32 pipe instead: Knuth's
// TwoSum, the FMA TwoProduct, and Dekker's double-length sum, product and
// quotient (Dekker 1971).  The rounded operations are written as intrinsics
// so that no contraction or fast-math rewrite can change them.
// ---------------------------------------------------------------------------
struct f2p {
  float h, l;
};
__device__ __forceinline__ f2p two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ f2p fast_two_sum(float a, float b) {  // |a| >= |b| or a = 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ f2p df_add(f2p a, f2p b) {
  const f2p s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ f2p df_mul(f2p a, f2p b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);  // a.h * b.h = p + e exactly
  e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));
  return fast_two_sum(p, e);
}
__device__ __forceinline__ f2p df_div(f2p a, f2p b) {
  const float r = __frcp_rn(b.h);
  const float q = __fmul_rn(a.h, r);
  const float p = __fmul_rn(q, b.h);
  const float pe = __fmaf_rn(q, b.h, -p);  // q * b.h = p + pe exactly
  // remainder a - q*b: a.h - p is exact (p is within a factor 2 of a.h)
  float rem = __fsub_rn(__fsub_rn(a.h, p), pe);
  rem = __fadd_rn(rem, __fmaf_rn(-q, b.l, a.l));
  return fast_two_sum(q, __fmul_rn(rem, r));
}
// x - d2f(x) as an FP32 number, by integer operations on the bits of x (no
// FP64 instruction).  d2f keeps the top 23 mantissa bits and rounds on the
// 29 it drops (D); the remainder is D * 2^(E-52), less 2^(E-23) when d2f
// rounded up, E the unbiased exponent of x.  It is formed exactly as
// F - B with B = 2^(E-23) and F = B * (1 + D / 2^29) (the 6 lowest bits of D
// truncated: 2^-46 relative to x).  Zero when x is zero, non-finite, or so
// small (|x| < 2^-103) or large (beyond FP32) that the pair has no low part.
__device__ __forceinline__ float lo_part(double x) {
  const unsigned int hi = (unsigned int)__double2hiint(x), lo = (unsigned int)__double2loint(x);
  const unsigned int ex = (hi >> 20) & 0x7FFu;
  const unsigned int sg = hi & 0x80000000u;
  const unsigned int ef = (ex - 919u) << 23;  // FP32 exponent field of 2^(E-23)
  const float B = __uint_as_float(sg | ef);
  const float F = __uint_as_float(sg | ef | ((lo & 0x1FFFFFFFu) >> 6));
  float r = __fsub_rn(F, B);
  r = ((lo >> 28) & 1u) ? __fsub_rn(r, B) : r;
  return (ex < 920u || ex > 1150u) ? 0.0f : r;
}
__device__ __forceinline__ f2p split(double x) { return {d2f(x), lo_part(x)}; }

__device__ __forceinline__ float warp_maxf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// One cell of the primitive pass: state index from g, primitive index from
// gq (the primitive arrays' geometry; equal to g in 2D).  lS / lC
// accumulate the interior maxima of the wave speed and |C_hat| when `red`
// is set (reduced by the caller).  mu (3D viscous) receives the mixture
// viscosity sum_s Y_s mu_s.
//
// FP64 work is kept to what the pressure needs: the mixture heat capacities
// (gamma - 1 = sum rho_s R_s / sum rho_s cv_s) and p = (gamma-1)(E - KE).
// The kinetic energy is formed in FP32: its error (1e-7 KE) is below the
// FP32 flux error wherever KE matters and negligible where it does not (the
// near-hydrostatic states whose pressure gradient needs FP64 accuracy).
// The pressure goes out as FP64 (pr) or as an FP32 pair hi + lo (pp[q],
// pp[q + qv]) that carries ~48 bits: differences of neighbouring pressures
// then come out of FP32 arithmetic (hi - hi' is exact for close values).
template <int NDIM>
__device__ __forceinline__ void mprim_cell(const Geo& g, const Geo& gq, const Phys& P,
                                           const double* __restrict__ U, float* __restrict__ Q,
                                           float* __restrict__ rho, double* __restrict__ rho64,
                                           float* __restrict__ vel, double* __restrict__ pr,
                                           float* __restrict__ pp, float* __restrict__ mu,
                                           float* __restrict__ nrg, float* __restrict__ Cc,
                                           float* __restrict__ T, float* __restrict__ lo,
                                           bool red, int i, int j, int k, float& lS, float& lC) {
  const long long sv = g.sv, qv = gq.sv;
  const long long c = (long long)i + g.sy * j + g.sz * k;
  const long long q = (long long)i + gq.sy * j + gq.sz * k;
  const int s0 = NDIM + 1;  // first species index
  // mixture EOS (calculateRhoPT, src/secondary.hpp:60-151)
  // The species loop stays rolled: unrolling it (all loads issued up front)
  // measured 1.5x slower for this streaming pass on GB300, as did forming
  // the two sums in double-float on the FP32 pipe.
  double sCv = 0.0, sRm = 0.0, r64 = 0.0;
  float rf = 0.f;
  for (int s = 0; s < P.ns; ++s) {
    const double rs = U[c + sv * (s0 + s)];
    if (rho64) r64 += rs;
    sCv = fma(rs, P.cv_s[s], sCv);
    sRm = fma(rs, P.rm_s[s], sRm);
    rf += d2f(rs);
  }
  const float rif = __frcp_rn(rf);
  const double gm1 = sRm * rcp64(sCv);
  float Cv2 = 0.f, Cp2 = 0.f, m = 0.f;
  for (int s = 0; s < P.ns; ++s) {
    const float rs = d2f(U[c + sv * (s0 + s)]);
    const float ys = rs * rif;
    if (NDIM == 2) {
      Cv2 += ys * P.cv2_f[s];
      Cp2 += ys * P.cp2_f[s];
    }
    m += ys * P.mu_f[s];
    Q[q + qv * (s0 + s)] = rs;
  }
  if (mu) mu[q] = m;
  float msq = 0.f, usq = 0.f;
#pragma unroll
  for (int d = 0; d < NDIM; ++d) {
    const float mf = d2f(U[c + sv * d]);
    msq += mf * mf;
    const float u = mf * rif;
    usq += u * u;
    vel[q + qv * d] = u;
    Q[q + qv * d] = mf;
  }
  const double E = U[c + sv * NDIM];
  const double p = gm1 * (E - f2d(0.5f * msq * rif));  // FP64 pressure recovery
  if (pr) pr[q] = p;
  if (pp) {
    const float ph = d2f(p);
    pp[q] = ph;
    pp[q + qv] = d2f(p - f2d(ph));
  }
  Q[q + qv * NDIM] = d2f(E + p);
  rho[q] = rf;
  if (rho64) rho64[q] = r64;
  if (T) T[q] = d2f(p) / d2f(sRm);  // p / (rho R_mix), R_mix = sum rho_s R_s / rho
  if (nrg) nrg[q] = d2f(E) * rif - 0.5f * rf * usq;  // E/rho - 0.5*rho*|u|^2 (reference)
  if (lo) {
    // C-equation runs: rho, the velocity and nrg as FP32 pairs (high parts
    // replace the FP32 values above), for the shock and contact switches;
    // lo = [rho, nrg, u, v] low parts (see Prim3Out)
    f2p r = {0.f, 0.f};
    for (int s = 0; s < P.ns; ++s) r = df_add(r, split(U[c + sv * (s0 + s)]));
    f2p m2 = {0.f, 0.f};
#pragma unroll
    for (int d = 0; d < NDIM; ++d) {
      const f2p md = split(U[c + sv * d]);
      const f2p u = df_div(md, r);
      vel[q + qv * d] = u.h;
      lo[q + qv * (2 + d)] = u.l;
      m2 = df_add(m2, df_mul(md, md));
    }
    const f2p kq = df_div(m2, r);  // rho |u|^2
    const f2p e = df_add(df_div(split(E), r), f2p{-0.5f * kq.h, -0.5f * kq.l});
    rho[q] = r.h;
    lo[q] = r.l;
    nrg[q] = e.h;
    lo[q + qv] = e.l;
  }
  if (Cc)
    for (int n = 0; n < 5; ++n) Cc[q + qv * n] = d2f(U[c + sv * (P.nv + n)]);
  if (red) {
    const bool in = i >= g.ng && i < g.ngi - g.ng && j >= g.ng && j < g.ngj - g.ng &&
                    (NDIM == 2 || (k >= g.ng && k < g.ngk - g.ng));
    if (in) {
      const float pf = d2f(p), mf = sqrtf(msq);
      float sp;
      if (NDIM == 3) sp = sqrtf((1.0f + d2f(gm1)) * pf * rif) + mf * rif;
      else sp = sqrtf(Cp2 / Cv2 * pf * rif) + mf;  // maxWaveSpeed2D quirks
      lS = fmaxf(lS, sp);
      lC = fmaxf(lC, fabsf(Cc[q + qv]));
    }
  }
}

// Outputs of the 3D primitive pass (primitive layout gq).  lo, when set
// (C-equation runs), receives the low parts of five FP32 pairs: [0] rho,
// [1] the C-equation internal energy, [2..4] u, v, w; their high parts are
// rho, nrg and vel.  rho64 (buoyancy) receives the density as an FP64 value.
struct Prim3Out {
  float *Q, *rho, *vel, *pp, *mu, *nrg, *C, *lo;
  double* rho64;
};

// The 3D equation of state with no FP64 instruction, in FP32 pairs.  The
// state values enter as pairs (d2f + lo_part); the density rho = sum rho_s,
// the mixture sums sum rho_s cv_s and sum rho_s R_s, gamma - 1 = their
// quotient and p = (gamma-1)(E - KE) (calculateRhoPT3D,
// src/secondary.hpp:109-151) carry ~48 bits, the accuracy the pressure
// gradient needs where it is a small difference of large pressures.  KE is
// FP32, as in mprim_cell.  The velocity u = m/rho (computeVelocity3D,
// src/velocity.hpp:68-83) and the C-equation energy nrg = E/rho -
// 0.5*rho*|u|^2 (calculateRhoGrad, src/ceq3d.hpp:138-141; rho*|u|^2 formed as
// |m|^2/rho) are pairs as well: the shock and contact switches of updateCeq
// take the signs of products of their derivatives, and FP32 rounding of the
// values alone flips them wherever a derivative is small against the value.
//
// eos3: one cell from its FP64 state values (species us[0..ns), momenta
// um[0..2], energy um[3]), written to O at primitive index q (field stride
// qv); returns the cell's wave speed |u| + c in *sp.  NS: the species count
// when it is known at compile time (every loop then unrolls), 0 for any.
template <int NS>
__device__ __forceinline__ void eos3(const Phys& P, const double* us, const double um[4],
                                     const Prim3Out& O, long long q, long long qv, float* sp) {
  f2p r = {0.f, 0.f}, cv = {0.f, 0.f}, rm = {0.f, 0.f};
  float msum = 0.f;
  const int ns = NS > 0 ? NS : P.ns;
#pragma unroll
  for (int s = 0; s < (NS > 0 ? NS : FST_MAX_SPECIES); ++s) {
    if (NS == 0 && s >= ns) break;
    const f2p a = split(us[s]);
    O.Q[q + qv * (4 + s)] = a.h;
    r = df_add(r, a);
    cv = df_add(cv, df_mul(a, f2p{P.cv_f[s], P.cv_lf[s]}));
    rm = df_add(rm, df_mul(a, f2p{P.rm_f[s], P.rm_lf[s]}));
    msum = fmaf(a.h, P.mu_f[s], msum);
  }
  const float rif = __frcp_rn(r.h);
  if (O.mu) O.mu[q] = msum * rif;  // sum_s Y_s mu_s
  f2p m[3];
  float msq = 0.f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    m[d] = split(um[d]);
    O.Q[q + qv * d] = m[d].h;
    msq = fmaf(m[d].h, m[d].h, msq);
    const f2p u = df_div(m[d], r);
    O.vel[q + qv * d] = u.h;
    if (O.lo) O.lo[q + qv * (2 + d)] = u.l;
  }
  const f2p E = split(um[3]);
  const f2p gm1 = df_div(rm, cv);
  const f2p p = df_mul(gm1, df_add(E, f2p{-0.5f * msq * rif, 0.f}));
  O.pp[q] = p.h;
  O.pp[q + qv] = p.l;
  O.Q[q + qv * 3] = E.h + p.h;  // E + p, the energy's advected quantity
  O.rho[q] = r.h;
  if (O.rho64) O.rho64[q] = f2d(r.h) + f2d(r.l);
  if (O.nrg) {
    f2p m2 = df_mul(m[0], m[0]);
    m2 = df_add(m2, df_mul(m[1], m[1]));
    m2 = df_add(m2, df_mul(m[2], m[2]));
    const f2p kq = df_div(m2, r);  // rho |u|^2
    const f2p e = df_add(df_div(E, r), f2p{-0.5f * kq.h, -0.5f * kq.l});
    O.nrg[q] = e.h;
    if (O.lo) {
      O.lo[q] = r.l;
      O.lo[q + qv] = e.l;
    }
  }
  *sp = sqrtf((1.0f + gm1.h) * p.h * rif) + sqrtf(msq) * rif;
}

// One cell of the 3D primitive pass from its FP64 state values (species
// us[0..ns), momenta and energy um[0..3], C variables uc[0..4] when O.C):
// writes the equation of state (eos3) and the FP32 C variables, and
// accumulates the interior maxima of the wave speed and |C_hat| when `red`
// is set.
template <int NS>
__device__ __forceinline__ void mprim3_vals(const Geo& g, const Phys& P, const double* us,
                                            const double um[4], const double uc[5],
                                            const Prim3Out& O, long long q, long long qv,
                                            bool red, int i, int j, int k, float& lS, float& lC) {
  float sp;
  eos3<NS>(P, us, um, O, q, qv, &sp);
  if (O.C) {
#pragma unroll
    for (int n = 0; n < 5; ++n) O.C[q + qv * n] = d2f(uc[n]);
  }
  if (red) {
    const bool in = i >= g.ng && i < g.ngi - g.ng && j >= g.ng && j < g.ngj - g.ng &&
                    k >= g.ng && k < g.ngk - g.ng;
    if (in) {
      lS = fmaxf(lS, sp);
      lC = fmaxf(lC, fabsf(d2f(uc[1])));
    }
  }
}

// mprim3_vals of cell (i, j, k) of U, every value loaded before any is used
// (a thread has all its loads in flight at once).
template <int NS>
__device__ __forceinline__ void mprim3_cell(const Geo& g, const Geo& gq, const Phys& P,
                                            const double* __restrict__ U, const Prim3Out& O,
                                            bool red, int i, int j, int k, float& lS, float& lC) {
  const long long sv = g.sv, qv = gq.sv;
  const long long c = (long long)i + g.sy * j + g.sz * k;
  const long long q = (long long)i + gq.sy * j + gq.sz * k;
  double us[NS > 0 ? NS : FST_MAX_SPECIES], um[4], uc[5];
#pragma unroll
  for (int s = 0; s < (NS > 0 ? NS : FST_MAX_SPECIES); ++s) {
    if (NS == 0 && s >= P.ns) break;
    us[s] = U[c + sv * (4 + s)];
  }
#pragma unroll
  for (int d = 0; d < 4; ++d) um[d] = U[c + sv * d];
  if (O.C) {
#pragma unroll
    for (int n = 0; n < 5; ++n) uc[n] = U[c + sv * (P.nv + n)];
  }
  mprim3_vals<NS>(g, P, us, um, uc, O, q, qv, red, i, j, k, lS, lC);
}

// ---------------------------------------------------------------------------
// FP32 WENO5-JS with the reference's weights (src/flux.hpp:241-266),
// rearranged for fewer operations and less rounding:
//  - with d_m = f_m - f_{m+1}, every smoothness indicator is
//    (13/12) a^2 + (1/4) b^2 with a, b short combinations of the d_m; all
//    three are taken x4 as (13/3) a^2 + b^2 with eps x4, which leaves the
//    normalised weights unchanged;
//  - the nonlinear weights are scaled by the smallest (eps+beta), so that no
//    square overflows or underflows in FP32;
//  - the candidate polynomials are p_k = f3 + q_k/6 (q_k in the d_m), so the
//    result is f3 + sum(w_k q_k) / (6 sum w_k): a correction to f3.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float weno_f(float f1, float f2, float f3, float f4, float f5) {
  const float d1 = f1 - f2, d2 = f2 - f3, d3 = f3 - f4, d4 = f4 - f5;
  const float c = 13.0f / 3.0f, eps = 4.0e-6f;
  float a = d1 - d2, b = d1 - 3.0f * d2;  // f1-2f2+f3, f1-4f2+3f3
  const float e1 = eps + (c * a * a + b * b);
  a = d2 - d3;                            // f2-2f3+f4
  b = d2 + d3;                            // f2-f4
  const float e2 = eps + (c * a * a + b * b);
  a = d3 - d4;                            // f3-2f4+f5
  b = 3.0f * d3 - d4;                     // 3f3-4f4+f5
  const float e3 = eps + (c * a * a + b * b);
  const float mn = fminf(e1, fminf(e2, e3));
  const float r1 = __fdividef(mn, e1), r2 = __fdividef(mn, e2), r3 = __fdividef(mn, e3);
  const float s1 = r1 * r1, s2 = r2 * r2, s3 = r3 * r3;
  // d_k q_k with d = (0.1, 0.6, 0.3): q1 = 2d1-5d2, q2 = -d2-2d3, q3 = d4-4d3
  const float num = s1 * (0.2f * d1 - 0.5f * d2) + s2 * (-0.6f * d2 - 1.2f * d3) +
                    s3 * (0.3f * d4 - 1.2f * d3);
  const float den = 0.6f * s1 + 3.6f * s2 + 1.8f * s3;  // 6 sum d_k s_k
  return f3 + __fdividef(num, den);
}

// The linear 5th-order upwind reconstruction: WENO5 with the optimal weights
// d = (0.1, 0.6, 0.3), i.e. (2 f1 - 13 f2 + 47 f3 + 27 f4 - 3 f5) / 60.
__device__ __forceinline__ float upwind5_f(float f1, float f2, float f3, float f4, float f5) {
  return (1.0f / 30.0f) * f1 + (-13.0f / 60.0f) * f2 + (47.0f / 60.0f) * f3 +
         (27.0f / 60.0f) * f4 + (-1.0f / 20.0f) * f5;
}

struct FaceCtx {
  float rd[3];   // 1/dx, 1/dy, 1/dz
  float r4d[3];  // 1/(4dx) ...
  float alpha;
};

__device__ __forceinline__ FaceCtx make_ctx(const Phys& P, const unsigned long long* red,
                                            float* maxS) {
  FaceCtx fc;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    fc.rd[d] = P.rd_f[d];
    fc.r4d[d] = 0.25f * P.rd_f[d];
  }
  fc.alpha = 0.f;
  *maxS = 0.f;
  if (P.ceq) {
    const float maxCh = d2f(fst_unkey(red[1]));
    fc.alpha = P.dxmag2_f / (maxCh + 1.0e-6f) * P.alpha_f;  // src/cart3d.cpp:285
    *maxS = d2f(fst_unkey(red[0]));
  }
  return fc;
}

__device__ __forceinline__ bool smooth_at(const unsigned char* map, long long c, int f) {
  return map != nullptr && map[c * 3 + f] != 0;
}

// ---------------------------------------------------------------------------
// 2D face terms of cart2d (src/flux.hpp:23-106, src/viscosity.hpp:25-199,
// src/ceq.hpp:200-293) with their quirks, in FP32.
// ---------------------------------------------------------------------------
template <int NV, bool HYB>
__device__ __forceinline__ void face2d(const Geo& g, const Phys& P, const MixedView& M,
                                       const FaceCtx& fc, long long c, int f, bool smooth,
                                       int nv, float* G) {
  const long long sv = g.sv, sx = 1, sy = g.sy;
  const long long sf = f == 0 ? sx : sy;
  const float* un = M.vel + sv * f;
  const float uf = (-un[c + 2 * sf] + 7.0f * un[c + sf] + 7.0f * un[c] - un[c - sf]) * (1.0f / 12.0f);
  const bool neg = uf < 0.0f;
  const long long c0 = neg ? c + 3 * sf : c - 2 * sf;
  const long long o = neg ? -sf : sf;
  const float scale = uf * fc.rd[f];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    if (NV == NVMAX && v >= nv) break;
    const float* q = M.Q + sv * v;
    const float f1 = __ldg(q + c0), f2 = __ldg(q + c0 + o), f3 = __ldg(q + c0 + 2 * o),
                f4 = __ldg(q + c0 + 3 * o), f5 = __ldg(q + c0 + 4 * o);
    G[v] = scale * ((HYB && smooth) ? upwind5_f(f1, f2, f3, f4, f5) : weno_f(f1, f2, f3, f4, f5));
  }
  if (!(P.visc || P.ceq)) return;
  const float* u = M.vel;
  const float* v = M.vel + sv;
  float V[3] = {0.f, 0.f, 0.f};  // x-, y-momentum, energy
  if (P.visc) {
    const float mu = P.mu2d_f;
    float dudx, dvdx, dudy, dvdy;
    if (f == 0) {
      dudx = (u[c + sx] - u[c]) * fc.rd[0];
      dvdx = (v[c + sx] - v[c]) * fc.rd[0];
      dudy = ((u[c + sy] + u[c + sx + sy]) - (v[c - sy] + u[c + sx - sy])) * fc.r4d[1];  // vel(i,j-1,1)
      dvdy = ((v[c + sy] + v[c + sx + sy]) - (v[c - sy] + v[c + sx - sy])) * fc.r4d[1];
    } else {
      dudx = ((u[c + sx] + u[c + sx + sy]) - (u[c - sx] + u[c - sx + sy])) * fc.r4d[0];
      dvdx = ((v[c + sx] + v[c + sx + sy]) - (v[c - sx] + v[c - sx + sy])) * fc.r4d[0];
      dudy = (u[c + sy] - u[c]) * fc.rd[1];
      dvdy = (v[c + sy] - v[c]) * fc.rd[1];
    }
    const float sxx = (2.0f / 3.0f) * mu * (2.0f * dudx - dvdy);
    const float syy = (2.0f / 3.0f) * mu * (2.0f * dvdy - dudx);
    const float sxy = mu * (dudy + dvdx);
    const float sn = f == 0 ? sxx : sxy;  // x-momentum component on this face
    const float st = f == 0 ? sxy : syy;  // y-momentum component
    const float q = -P.kheat_f * (M.T[c + sf] - M.T[c]) * fc.rd[f];
    V[0] = sn;
    V[1] = st;
    V[2] = 0.5f * (u[c + sf] + u[c]) * sn + 0.5f * (v[c + sf] + v[c]) * st - q;
  }
  if (P.ceq) {
    const float r = 0.5f * (M.rho[c] + M.rho[c + sf]);
    const float chat = 0.5f * (M.C[c + sv] + M.C[c + sf + sv]);
    const float ct0 = 0.5f * (M.C[c + 2 * sv] + M.C[c + sf + 2 * sv]);
    const float ct1 = 0.5f * (M.C[c + 3 * sv] + M.C[c + sf + 3 * sv]);
    const float rct = __fdividef(1.0f, ct0 * ct0 + ct1 * ct1 + 1.0e-6f);
    const float ctf = f == 0 ? ct0 : ct1;
    const float arc = fc.alpha * r * chat * ctf * rct;
#pragma unroll
    for (int w = 0; w < 2; ++w) {
      const float* vw = M.vel + sv * w;
      float g0, g1;
      if (f == 0) {
        g0 = (vw[c + sx] - vw[c]) * fc.rd[0];
        g1 = ((vw[c + sy] + vw[c + sx + sy]) - (vw[c - sy] + vw[c + sx - sy])) * fc.r4d[1];
      } else {
        g0 = ((vw[c + sx] + vw[c + sx + sy]) - (vw[c - sx] + vw[c - sx + sy])) * fc.r4d[0];
        g1 = (vw[c + sy] - vw[c]) * fc.rd[1];
      }
      V[w] += arc * (ct0 * g0 + ct1 * g1);
    }
  }
  G[0] -= V[0] * fc.rd[f];
  G[1] -= V[1] * fc.rd[f];
  G[2] -= V[2] * fc.rd[f];
}

// One TXX x TYY thread tile of the fused 2D RHS + RK stage (tile (bx, by)
// of the case; TXX = 16, 32 or 64 threads along i).  sG is the block's
// shared staging of the y faces; the x face left of a cell comes from the
// neighbouring lane by shuffle (within TXX lanes when TXX < 32), and for
// TXX = 64 the first lane of the second warp of a row reads it from sE,
// where the last lane of the first warp left it.  All threads of the block
// must call it (it synchronises).
template <int NV, bool HYB, int TYY, int TXX = TX>
__device__ __forceinline__ void rhs2d_tile(const Geo& g, const Phys& P, const MixedView& M,
                                           const unsigned long long* __restrict__ red,
                                           const unsigned char* __restrict__ smap,
                                           const double* Uold, double* Unew, double coef,
                                           double* __restrict__ Rout, int bx, int by,
                                           float (*sG)[TXX][NV], float (*sE)[NV] = nullptr) {
  static_assert(TXX == 16 || TXX == 32 || TXX == 64, "tile width 16, 32 or 64");
  constexpr int kWarpsX = TXX > 32 ? TXX / 32 : 1;
  constexpr int kShflW = TXX < 32 ? TXX : 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i = g.ng - 1 + bx * (TXX - 1) + tx;
  const int j = g.ng - 1 + by * (TYY - 1) + ty;
  const long long sv = g.sv, sy = g.sy;
  const int nv = P.nv;
  float maxS;
  FaceCtx fc = make_ctx(P, red, &maxS);
  fc.rd[2] = fc.rd[0];
  const bool fi = i <= g.ngi - g.ng - 1;
  const bool fj = j <= g.ngj - g.ng - 1;
  const bool ci = tx >= 1 && i >= g.ng && i < g.ngi - g.ng;
  const bool cj = ty >= 1 && j >= g.ng && j < g.ngj - g.ng;
  const long long c = (long long)i + sy * j;
  float Gx[NV], Gy[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) Gx[v] = Gy[v] = 0.f;
  if (fi && cj) face2d<NV, HYB>(g, P, M, fc, c, 0, HYB && smooth_at(smap, c, 0), nv, Gx);
  if (fj && ci) face2d<NV, HYB>(g, P, M, fc, c, 1, HYB && smooth_at(smap, c, 1), nv, Gy);
#pragma unroll
  for (int v = 0; v < NV; ++v) sG[ty][tx][v] = Gy[v];
  if (kWarpsX > 1 && (tx & 31) == 31) {
#pragma unroll
    for (int v = 0; v < NV; ++v) sE[ty * kWarpsX + (tx >> 5)][v] = Gx[v];
  }
  __syncthreads();
  const bool edge = kWarpsX > 1 && (tx & 31) == 0 && tx > 0;
  float R[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    float gxl = __shfl_up_sync(0xffffffffu, Gx[v], 1, kShflW);
    if (edge) gxl = sE[ty * kWarpsX + (tx >> 5) - 1][v];
    R[v] = 0.f;
    if (ci && cj) R[v] = -((Gx[v] - gxl) + (Gy[v] - sG[ty - 1][tx][v]));
  }
  if (!(ci && cj)) return;
  const double* p = M.p;
  const double dpx = (p[c - 2] - 8.0 * p[c - 1] + 8.0 * p[c + 1] - p[c + 2]) * P.r12x;
  const double dpy = (p[c - 2 * sy] - 8.0 * p[c - sy] + 8.0 * p[c + sy] - p[c + 2 * sy]) * P.r12y;
  double Rd[3] = {f2d(R[0]) - dpx, f2d(R[1]) - dpy, f2d(R[2])};
  if (P.buoyancy) {
    const double rhop = M.rho64[c] - P.rho_ref;
    if (rhop >= 1e-6 || rhop <= -1e-6) {
      const double f = -P.g * rhop;
      const float vb = M.Q[c + sv] / M.Q[c + 3 * sv];  // m_y / rho_1 (reference)
      Rd[1] += f;
      Rd[2] += f2d(fabsf(vb)) * f;
    }
  }
  auto emit = [&](int v, double Rv) {
    if (Rout) Rout[c + sv * v] = Rv;
    else Unew[c + sv * v] = Uold[c + sv * v] + coef * Rv;
  };
#pragma unroll
  for (int w = 0; w < 3; ++w) emit(w, Rd[w]);
#pragma unroll
  for (int v = 3; v < NV; ++v) {
    if (NV == NVMAX && v >= nv) break;
    emit(v, f2d(R[v]));
  }
  if (P.ceq) {
    const float r12x = P.r12_f[0], r12y = P.r12_f[1];
    // the switches take the signs of div u and grad rho . grad e: rho, e and
    // the velocity enter as FP32 pairs (high parts M.rho / M.nrg / M.vel,
    // low parts M.lo), differenced high with high and low with low
    auto d4 = [&](const float* a, const float* l, long long st, float r12) {
      const float d1 = (a[c + st] - a[c - st]) + (l[c + st] - l[c - st]);
      const float d2 = (a[c + 2 * st] - a[c - 2 * st]) + (l[c + 2 * st] - l[c - 2 * st]);
      return (8.0f * d1 - d2) * r12;
    };
    const float* lo = M.lo;
    const float dxr = d4(M.rho, lo, 1, r12x), dyr = d4(M.rho, lo, sy, r12y);
    const float dxe = d4(M.nrg, lo + sv, 1, r12x), dye = d4(M.nrg, lo + sv, sy, r12y);
    const float divu = d4(M.vel, lo + 2 * sv, 1, r12x) + d4(M.vel + sv, lo + 3 * sv, sy, r12y);
    const float rgrad = sqrtf(dxr * dxr + dyr * dyr);
    const float dnednr = (dxr * dxe + dyr * dye) * (dxr * dxr + dyr * dyr);
    const bool i1 = dnednr < 0.0f;
    const float Gs[4] = {(!i1 && divu < 0.f) ? rgrad : 0.f, i1 ? rgrad : 0.f, -dyr, dxr};
    const float dxm = P.dxmag_f;
    const float src = maxS / (P.eps_f * dxm);
    const float dif = P.kap_f * maxS * dxm;
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      const float* Cn = M.C + sv * n;
      const float cc = Cn[c];
      const float lap = (Cn[c + 1] - 2.0f * cc + Cn[c - 1]) * fc.rd[0] +
                        (Cn[c + sy] - 2.0f * cc + Cn[c - sy]) * fc.rd[1];
      emit(nv + n, f2d(src * (Gs[n] - cc) + dif * lap));
    }
    emit(nv + 4, 0.0);
  }
}

}  // namespace fstm
