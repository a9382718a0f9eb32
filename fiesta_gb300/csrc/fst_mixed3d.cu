// fst_mixed3d.cu — the 3D mixed-precision (FST_MODE_MIXED) and learned-hybrid
// (FST_MODE_HYBRID) right-hand side + RK stage for sm_103a.
//
// Four 2.5D stencil kernels per stage, each updating its own conserved
// variables of U_new = U_old + coef*R in FP64 (R never goes to HBM):
//
//   k_mcell3d  the cell-centred terms of the momenta and energy: the
//              FP64-accurate pressure gradient (src/presgrad.hpp:41-74) and
//              buoyancy (src/buoyancy.hpp), U_new = U_old + coef*R_cell
//   k_mceq3d   the five C-equation variables (calculateRhoGrad, updateCeq,
//              src/ceq3d.hpp:95-224)
//   k_mspec3d  species densities: WENO5 advection, their only term
//   k_mmom3d   momenta and energy: WENO5 advection, the viscous stress
//              (calculateStressTensor{x,y,z}3dv, src/viscosity.hpp) and the
//              C-equation tensor terms (calculateCeqFaces/Grads, applyCeq,
//              src/ceq3d.hpp) of every face, added to what k_mcell3d wrote:
//              U_new += coef*R_face
//
// Splitting by variable keeps each kernel's z-window small enough for
// registers and its global loads few; the cost is reading the velocities
// three times and the momenta/energy of U_new twice.
//
// Face kernels: blocks of 32x8 threads march along k (16 planes).  Thread
// (tx, ty) owns column (i0-1+tx, j0-1+ty); it computes the face at i+1/2
// from the x-stencil, the face at j+1/2 from the y-stencil and, for the
// 31x7 interior columns, the face at k+1/2; the left x face comes from
// lane-1 by shuffle, the lower y face through shared memory, the back z face
// from the previous plane in registers, so every face is computed once.
//
// Plane data come in by TMA: one elected thread issues cp.async.bulk.tensor
// 4D copies of a 40x13 (x, y) box of consecutive fields -- the columns plus
// the 3-cell stencil halo, x rounded down to a multiple of 4 floats -- into
// shared memory.  Plane tiles are triple-buffered (plane k+2 is requested
// while plane k is computed) and the momentum kernel keeps a 5-slot ring of
// velocity planes (k-2 .. k+2) for the tangential derivatives, so one block
// barrier per plane covers both the y-face exchange (double-buffered) and
// the reuse of the oldest buffer.  The z-stencils come from register
// windows over the thread's own column, refilled by one coalesced load per
// variable per plane, one plane ahead; so is the old state.  Every mbarrier
// wait is bounded (fst_tma.cuh); a wait that runs out sets the context's
// device error word and the block returns after draining its copies.
//
// The equations, quirks included, are the reference's; only the precision
// differs (FP32 fluxes, FP64 state, pressure gradient and RK combine).
#include <cudaTypedefs.h>

#include "fst_mixed_dev.cuh"
#include "fst_tma.cuh"

struct Mixed3DMaps {
  CUtensorMap qs;   // Q, box of NSC species fields
  CUtensorMap q4;   // Q, box of fields 0..3 (momenta, E + p)
  CUtensorMap v2;   // velocity, box of u, v
  CUtensorMap v3;   // velocity, box of u, v, w
  CUtensorMap rho;  // FP32 density
  CUtensorMap nrg;  // C-equation internal energy
  CUtensorMap mu;   // mixture viscosity
  CUtensorMap c5;   // C-variables 0..4
  CUtensorMap c4;   // C-variables 1..4 (C_hat, C_1..3)
  CUtensorMap p;    // pressure hi/lo pair (2 FP32 fields)
  CUtensorMap lo4;  // pair low parts 0..3 (rho, e, u, v)
  int nsc;          // species per k_mspec3d launch
};

namespace {
using namespace fstm;
using namespace fsttma;

constexpr int HX = 40, HY = 13, PL = HX * HY;  // one field of a plane tile (floats)
constexpr int KZ3 = 16;                        // planes per block along k
constexpr int NBUF = 3;                        // plane tiles in flight per block
constexpr int NRING = 5;                       // velocity planes k-2 .. k+2

__host__ __device__ constexpr int al32(int n) { return (n + 31) & ~31; }  // 128-byte multiples

// Face-kernel placement: thread (tx, ty) owns column i = ng-1 + 31 bx + tx
// and row j = ng-1 + 7 by + ty.  The tile starts at x0 = (i_lane0 - 2)
// rounded down to a multiple of 4 (a TMA box must start on a 16-byte
// boundary) and at y0 = j_row0 - 2; with ng = 3 both are >= 0.  own: the
// thread's cell in the tile; its stencils span columns own-2 .. own+3
// (<= 39) and rows -2 .. +3 (<= 12).
struct Place {
  int i, j, x0, y0, own;
};
__device__ __forceinline__ Place place_faces(const Geo& g) {
  Place p;
  const int ib = g.ng - 1 + (TX - 1) * (int)blockIdx.x;
  const int jb = g.ng - 1 + (TY - 1) * (int)blockIdx.y;
  p.i = ib + (int)threadIdx.x;
  p.j = jb + (int)threadIdx.y;
  p.x0 = (ib - 2) & ~3;
  p.y0 = jb - 2;
  p.own = (p.j - p.y0) * HX + (p.i - p.x0);
  return p;
}
// Cell-kernel placement: 32x8 interior cells per block, i = ng + 32 bx + tx;
// stencils span +-2, i.e. columns own-2 .. own+2 <= 36, rows 0 .. 12.
__device__ __forceinline__ Place place_cells(const Geo& g) {
  Place p;
  const int ib = g.ng + TX * (int)blockIdx.x;
  const int jb = g.ng + TY * (int)blockIdx.y;
  p.i = ib + (int)threadIdx.x;
  p.j = jb + (int)threadIdx.y;
  p.x0 = (ib - 2) & ~3;
  p.y0 = jb - 2;
  p.own = (p.j - p.y0) * HX + (p.i - p.x0);
  return p;
}

// ---------------------------------------------------------------------------
// WENO5 of one face from five stencil values read at base + m*o, m = 0..4
// ---------------------------------------------------------------------------
template <bool HYB>
__device__ __forceinline__ float rec5(const float* q, int base, int o, bool smooth) {
  const float f1 = q[base], f2 = q[base + o], f3 = q[base + 2 * o], f4 = q[base + 3 * o],
              f5 = q[base + 4 * o];
  return (HYB && smooth) ? upwind5_f(f1, f2, f3, f4, f5) : weno_f(f1, f2, f3, f4, f5);
}
template <bool HYB>
__device__ __forceinline__ float rec5z(const float w[6], bool neg, bool smooth) {
  // window w[m] = plane k-2+m; upwind side by the sign of the face velocity
  const float f1 = neg ? w[5] : w[0], f2 = neg ? w[4] : w[1], f3 = neg ? w[3] : w[2],
              f4 = neg ? w[2] : w[3], f5 = neg ? w[1] : w[4];
  return (HYB && smooth) ? upwind5_f(f1, f2, f3, f4, f5) : weno_f(f1, f2, f3, f4, f5);
}
__device__ __forceinline__ float face_u(float um1, float u0, float u1, float u2) {
  return (-u2 + 7.0f * u1 + 7.0f * u0 - um1) * (1.0f / 12.0f);
}

// ---------------------------------------------------------------------------
// shared-memory layouts (offsets in floats; every TMA destination 128-byte
// aligned; mbarriers in the first 128 bytes)
// ---------------------------------------------------------------------------
constexpr int BAR_BYTES = 128;
constexpr int ALIGN_SLACK = 128;  // room to align the dynamic shared memory base

struct SpecLayout {
  int q, v, size;
  uint32_t bytes;  // TMA bytes per plane
};
__host__ __device__ inline SpecLayout spec_layout(int nsc) {
  SpecLayout L;
  L.q = 0;
  L.v = al32(nsc * PL);
  L.size = al32(L.v + 2 * PL);
  L.bytes = (uint32_t)((nsc + 2) * PL * 4);
  return L;
}
struct MomLayout {
  int q, mu, rho, c, tsize, rsize;
  uint32_t tbytes, rbytes;
};
__host__ __device__ inline MomLayout mom_layout(bool visc, bool ceq) {
  MomLayout L;
  L.q = 0;
  L.mu = al32(4 * PL);
  L.rho = al32(L.mu + PL);
  L.c = al32(L.rho + PL);
  L.tsize = al32(L.c + 4 * PL);
  L.rsize = al32(3 * PL);
  L.tbytes = (uint32_t)((4 + (visc ? 1 : 0) + (ceq ? 5 : 0)) * PL * 4);
  L.rbytes = (uint32_t)(3 * PL * 4);
  return L;
}
struct CellLayout {
  int p, v, size;  // p: pressure hi plane then lo plane; v: u, v
  uint32_t bytes;
};
__host__ __device__ inline CellLayout cell_layout() {
  CellLayout L;
  L.p = 0;
  L.v = al32(2 * PL);
  L.size = al32(L.v + 2 * PL);
  L.bytes = (uint32_t)(4 * PL * 4);
  return L;
}
struct CeqLayout {
  int v, rho, nrg, c, lo, size;  // lo: pair low parts of rho, e, u, v
  uint32_t bytes;
};
__host__ __device__ inline CeqLayout ceq_layout() {
  CeqLayout L;
  L.v = 0;
  L.rho = al32(2 * PL);
  L.nrg = al32(L.rho + PL);
  L.c = al32(L.nrg + PL);
  L.lo = al32(L.c + 5 * PL);
  L.size = al32(L.lo + 4 * PL);
  L.bytes = (uint32_t)(13 * PL * 4);
  return L;
}

__device__ __forceinline__ unsigned char* aligned_smem(unsigned char* p) {
  return p + ((128u - (smem_u32(p) & 127u)) & 127u);
}

// ---------------------------------------------------------------------------
// k_mcell3d: pressure gradient and buoyancy of the momenta and energy
// k_mceq3d:  the five C-equation variables (updateCeq)
// ---------------------------------------------------------------------------
// Fourth-order central derivative of an FP32-pair field from its high parts
// h and low parts l at offsets -2o .. 2o: the differences of neighbouring
// high parts are exact for close values and carry the low parts, so the
// result has FP32 accuracy relative to the derivative itself, not to the
// field's values.
__device__ __forceinline__ float d4pair(const float* h, const float* l, int o, float r12) {
  const float d1 = (h[o] - h[-o]) + (l[o] - l[-o]);
  const float d2 = (h[2 * o] - h[-2 * o]) + (l[2 * o] - l[-2 * o]);
  return (8.0f * d1 - d2) * r12;
}
// the same along z from 5-plane windows (w[m] = plane k-2+m)
__device__ __forceinline__ float d4pairz(const float h[5], const float l[5], float r12) {
  const float d1 = (h[3] - h[1]) + (l[3] - l[1]);
  const float d2 = (h[4] - h[0]) + (l[4] - l[0]);
  return (8.0f * d1 - d2) * r12;
}

__global__ void __launch_bounds__(TX * TY, 3)
    k_mcell3d(const __grid_constant__ Mixed3DMaps maps, Geo g, Geo gq, Phys P, MixedView M,
              const double* Uold, double* Unew, double coef, double* __restrict__ Rout,
              unsigned int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smdyn[];
  unsigned char* smraw = aligned_smem(smdyn);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw);
  const bool buoy = P.buoyancy != 0;
  const CellLayout L = cell_layout();
  float* tiles = reinterpret_cast<float*>(smraw + BAR_BYTES);
  const int tid = threadIdx.y * TX + threadIdx.x;
  const Place pl = place_cells(g);
  const int i = pl.i, j = pl.j;
  const int kc0 = g.ng + (int)blockIdx.z * KZ3;
  const int kc1 = min(kc0 + KZ3, g.ngk - g.ng);
  const bool cell = i < g.ngi - g.ng && j < g.ngj - g.ng;
  const long long cq0 = (long long)i + gq.sy * j;
  const long long c0 = (long long)i + g.sy * j;
  const long long sz = gq.sz;
  if (tid == 0) {
    prefetch_map(&maps.p);
    prefetch_map(&maps.v2);
    for (int q = 0; q < NBUF; ++q) mbar_init(&bar[q], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int m) {  // plane kc0 + m into buffer m % NBUF
    const int buf = m % NBUF, k = kc0 + m;
    float* tb = tiles + buf * L.size;
    mbar_arrive_expect_tx(&bar[buf], L.bytes);
    tma_load_4d(tb + L.p, &maps.p, &bar[buf], pl.x0, pl.y0, k, 0);
    tma_load_4d(tb + L.v, &maps.v2, &bar[buf], pl.x0, pl.y0, k, 0);
  };
  if (tid == 0) {
    issue(0);
    if (kc0 + 1 < kc1) issue(1);
  }
  // own-column window of the pressure pair at planes k-2 .. k+2 (+ next)
  const float* plo = M.pp + gq.sv;
  float ph[5], pl5[5], phn = 0.f, pln = 0.f;
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    const long long o = cq0 + sz * (kc0 - 3 + m);  // planes kc0-3 .. kc0+1, shifted in below
    ph[m] = cell ? M.pp[o] : 0.f;
    pl5[m] = cell ? plo[o] : 0.f;
  }
  if (cell) {
    phn = M.pp[cq0 + sz * (kc0 + 2)];
    pln = plo[cq0 + sz * (kc0 + 2)];
  }
  // old state of the momenta and energy, one plane ahead
  double uo[4], un[4];
  auto load_old = [&](int k, double* u) {
    const long long c = c0 + g.sz * k;
#pragma unroll
    for (int w = 0; w < 4; ++w) u[w] = Uold[c + g.sv * w];
  };
  if (cell && !Rout) load_old(kc0, un);

  bool ok = true;
  int k = kc0;
  for (; k < kc1; ++k) {
    const int n = k - kc0, b = n % NBUF;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      ph[m] = ph[m + 1];
      pl5[m] = pl5[m + 1];
    }
    ph[4] = phn;
    pl5[4] = pln;
#pragma unroll
    for (int w = 0; w < 4; ++w) uo[w] = un[w];
    if (cell && k + 1 < kc1) {
      phn = M.pp[cq0 + sz * (k + 3)];
      pln = plo[cq0 + sz * (k + 3)];
      if (!Rout) load_old(k + 1, un);
    }
    ok = ok && mbar_wait(&bar[b], (uint32_t)((n / NBUF) & 1), err);
    if (cell && ok) {
      const float* tb = tiles + b * L.size;
      // 4th-order pressure gradient (src/presgrad.hpp:44-71) from the hi/lo
      // pair; reference quirk: the z spacing is dy
      const float* th = tb + L.p + pl.own;
      const float* tl = th + PL;
      const float dpx = d4pair(th, tl, 1, P.r12_f[0]);
      const float dpy = d4pair(th, tl, HX, P.r12_f[1]);
      const float dpz = d4pairz(ph, pl5, P.r12_f[1]);
      double Rd[4] = {-f2d(dpx), -f2d(dpy), -f2d(dpz), 0.0};
      if (buoy) {  // computeBuoyancy3D (src/buoyancy.hpp:22-47)
        const float* tu = tb + L.v + pl.own;
        const double f = -P.g * (M.rho64[cq0 + sz * k] - P.rho_ref);
        Rd[1] += f;
        Rd[3] += f2d(tu[PL]) * f;
      }
      const long long c = c0 + g.sz * k;
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        if (Rout) Rout[c + g.sv * w] = Rd[w];
        else Unew[c + g.sv * w] = uo[w] + coef * Rd[w];
      }
    }
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    if (tid == 0 && k + 2 < kc1) {
      fence_proxy_async();
      issue(n + 2);
    }
  }
  if (!ok && tid == 0) {
    // a wait ran out: let the copies in flight land (bounded)
    for (int m = k - kc0; m <= k - kc0 + 1 && kc0 + m < kc1; ++m)
      mbar_wait(&bar[m % NBUF], (uint32_t)((m / NBUF) & 1), err);
  }
}

// calculateRhoGrad + updateCeq (src/ceq3d.hpp:95-224): the shock and contact
// switches take the signs of div u and of grad rho . grad e, so rho, e and
// the velocity enter as FP32 pairs (hi parts from rho, nrg, vel; lo parts
// from M.lo); the C variables and their Laplacian are FP32.  Cn (fused
// stages): the next stage's FP32 C variables of U_new and, in red_n[1], the
// interior maximum of |C_hat| of U_new.
__global__ void __launch_bounds__(TX * TY, 2)
    k_mceq3d(const __grid_constant__ Mixed3DMaps maps, Geo g, Geo gq, Phys P, MixedView M,
             const unsigned long long* __restrict__ red, const double* Uold, double* Unew,
             double coef, double* __restrict__ Rout, unsigned int* __restrict__ err,
             float* __restrict__ Cn, unsigned long long* __restrict__ red_n) {
  extern __shared__ __align__(128) unsigned char smdyn[];
  unsigned char* smraw = aligned_smem(smdyn);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw);
  const CeqLayout L = ceq_layout();
  float* tiles = reinterpret_cast<float*>(smraw + BAR_BYTES);
  const int tid = threadIdx.y * TX + threadIdx.x;
  const Place pl = place_cells(g);
  const int i = pl.i, j = pl.j;
  const int kc0 = g.ng + (int)blockIdx.z * KZ3;
  const int kc1 = min(kc0 + KZ3, g.ngk - g.ng);
  const bool cell = i < g.ngi - g.ng && j < g.ngj - g.ng;
  const long long cq0 = (long long)i + gq.sy * j;
  const long long c0 = (long long)i + g.sy * j;
  const long long sz = gq.sz, qv = gq.sv;
  float maxS;
  const FaceCtx fc = make_ctx(P, red, &maxS);
  if (tid == 0) {
    prefetch_map(&maps.rho);
    prefetch_map(&maps.lo4);
    for (int q = 0; q < NBUF; ++q) mbar_init(&bar[q], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int m) {  // plane kc0 + m into buffer m % NBUF
    const int buf = m % NBUF, k = kc0 + m;
    float* tb = tiles + buf * L.size;
    mbar_arrive_expect_tx(&bar[buf], L.bytes);
    tma_load_4d(tb + L.v, &maps.v2, &bar[buf], pl.x0, pl.y0, k, 0);
    tma_load_4d(tb + L.rho, &maps.rho, &bar[buf], pl.x0, pl.y0, k, 0);
    tma_load_4d(tb + L.nrg, &maps.nrg, &bar[buf], pl.x0, pl.y0, k, 0);
    tma_load_4d(tb + L.c, &maps.c5, &bar[buf], pl.x0, pl.y0, k, 0);
    tma_load_4d(tb + L.lo, &maps.lo4, &bar[buf], pl.x0, pl.y0, k, 0);
  };
  if (tid == 0) {
    issue(0);
    if (kc0 + 1 < kc1) issue(1);
  }
  // own-column windows at planes k-2 .. k+2 (+ next) of the pairs of rho, e
  // and w; C at k-1 .. k+1 (+ next)
  const float* vz = M.vel + 2 * qv;
  const float* rlo = M.lo;  // pair low parts: [0] rho, [1] e, [4] w
  const float* elo = M.lo + qv;
  const float* wlo = M.lo + 4 * qv;
  float rw[5], rl[5], ew[5], el[5], ww[5], wl[5];
  float rn = 0.f, rln = 0.f, en = 0.f, eln = 0.f, wn = 0.f, wln = 0.f;
  float cw[5][3], cn[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    const long long o = cq0 + sz * (kc0 - 3 + m);  // planes kc0-3 .. kc0+1, shifted in below
    rw[m] = cell ? M.rho[o] : 0.f;
    rl[m] = cell ? rlo[o] : 0.f;
    ew[m] = cell ? M.nrg[o] : 0.f;
    el[m] = cell ? elo[o] : 0.f;
    ww[m] = cell ? vz[o] : 0.f;
    wl[m] = cell ? wlo[o] : 0.f;
  }
  if (cell) {
    const long long o = cq0 + sz * (kc0 + 2);
    rn = M.rho[o];
    rln = rlo[o];
    en = M.nrg[o];
    eln = elo[o];
    wn = vz[o];
    wln = wlo[o];
  }
#pragma unroll
  for (int q = 0; q < 5; ++q) {
#pragma unroll
    for (int m = 0; m < 3; ++m) cw[q][m] = cell ? M.C[cq0 + qv * q + sz * (kc0 - 2 + m)] : 0.f;
    cn[q] = cell ? M.C[cq0 + qv * q + sz * (kc0 + 1)] : 0.f;
  }
  // old state of the C variables, one plane ahead
  double uo[5], un[5];
  auto load_old = [&](int k, double* u) {
    const long long c = c0 + g.sz * k;
#pragma unroll
    for (int q = 0; q < 5; ++q) u[q] = Uold[c + g.sv * (P.nv + q)];
  };
  if (cell && !Rout) load_old(kc0, un);
  float lC = -3.0e38f;

  bool ok = true;
  int k = kc0;
  for (; k < kc1; ++k) {
    const int n = k - kc0, b = n % NBUF;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      rw[m] = rw[m + 1];
      rl[m] = rl[m + 1];
      ew[m] = ew[m + 1];
      el[m] = el[m + 1];
      ww[m] = ww[m + 1];
      wl[m] = wl[m + 1];
    }
    rw[4] = rn;
    rl[4] = rln;
    ew[4] = en;
    el[4] = eln;
    ww[4] = wn;
    wl[4] = wln;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      cw[q][0] = cw[q][1];
      cw[q][1] = cw[q][2];
      cw[q][2] = cn[q];
      uo[q] = un[q];
    }
    if (cell && k + 1 < kc1) {
      const long long o = cq0 + sz * (k + 3);
      rn = M.rho[o];
      rln = rlo[o];
      en = M.nrg[o];
      eln = elo[o];
      wn = vz[o];
      wln = wlo[o];
#pragma unroll
      for (int q = 0; q < 5; ++q) cn[q] = M.C[cq0 + qv * q + sz * (k + 2)];
      if (!Rout) load_old(k + 1, un);
    }
    ok = ok && mbar_wait(&bar[b], (uint32_t)((n / NBUF) & 1), err);
    if (cell && ok) {
      const float* tb = tiles + b * L.size;
      const float r12x = P.r12_f[0], r12y = P.r12_f[1], r12z = P.r12_f[2];
      const float* tu = tb + L.v + pl.own;
      const float* tr = tb + L.rho + pl.own;
      const float* tn = tb + L.nrg + pl.own;
      const float* tlo = tb + L.lo + pl.own;  // rho, e, u, v low parts
      const float dxr = d4pair(tr, tlo, 1, r12x), dyr = d4pair(tr, tlo, HX, r12y);
      const float dzr = d4pairz(rw, rl, r12z);
      const float dxe = d4pair(tn, tlo + PL, 1, r12x), dye = d4pair(tn, tlo + PL, HX, r12y);
      const float dze = d4pairz(ew, el, r12z);
      const float divu = d4pair(tu, tlo + 2 * PL, 1, r12x) +
                         d4pair(tu + PL, tlo + 3 * PL, HX, r12y) + d4pairz(ww, wl, r12z);
      const float rg2 = dxr * dxr + dyr * dyr + dzr * dzr;
      const float rgrad = sqrtf(rg2);
      const float dnednr = (dxr * dxe + dyr * dye + dzr * dze) * rg2;
      const bool ind = dnednr < 0.0f;
      const float Gs[5] = {divu < 0.f && !ind ? rgrad : 0.f, ind ? rgrad : 0.f, dxr, dyr, dzr};
      const float dxm = P.dxmag_f;
      const float src = maxS / (P.eps_f * dxm);
      const float dif = P.kap_f * maxS * dxm;
      const long long c = c0 + g.sz * k;
#pragma unroll
      for (int q = 0; q < 5; ++q) {
        const float* tc = tb + L.c + q * PL + pl.own;
        const float cc = tc[0];
        const float lap = (tc[-1] - 2.0f * cc + tc[1]) * fc.rd[0] +
                          (tc[-HX] - 2.0f * cc + tc[HX]) * fc.rd[1] +
                          (cw[q][0] - 2.0f * cc + cw[q][2]) * fc.rd[2];
        const double Rv = f2d(src * (Gs[q] - cc) + dif * lap);
        const long long a = c + g.sv * (P.nv + q);
        if (Rout) {
          Rout[a] = Rv;
        } else {
          const double unew = uo[q] + coef * Rv;
          Unew[a] = unew;
          if (Cn) {  // the next stage's FP32 C variables and max |C_hat|
            const float cf = d2f(unew);
            Cn[cq0 + sz * k + qv * q] = cf;
            if (q == 1) lC = fmaxf(lC, fabsf(cf));
          }
        }
      }
    }
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    if (tid == 0 && k + 2 < kc1) {
      fence_proxy_async();
      issue(n + 2);
    }
  }
  if (Cn) {  // maxGradFunctor(var, nv+1) of U_new (src/ceq3d.hpp:82-93)
    lC = warp_maxf(lC);
    if ((tid & 31) == 0 && lC > -1e38f) atomicMax(&red_n[1], fst_key((double)lC));
  }
  if (!ok && tid == 0) {
    for (int m = k - kc0; m <= k - kc0 + 1 && kc0 + m < kc1; ++m)
      mbar_wait(&bar[m % NBUF], (uint32_t)((m / NBUF) & 1), err);
  }
}

// ---------------------------------------------------------------------------
// k_mspec3d: species [sb, sb+nsk)
// ---------------------------------------------------------------------------
// EPI (fused stages, all species in this launch): the kernel runs last in
// the stage and, per cell, also evaluates the equation of state of U_new
// (eos3: its new species from registers, momenta and energy as k_mmom3d left
// them) into the next stage's primitive set On, and the wave-speed maximum
// into red_n[0].
template <int NS, bool HYB, bool EPI>
__global__ void __launch_bounds__(TX * TY, EPI ? 2 : 3)
    k_mspec3d(const __grid_constant__ Mixed3DMaps maps, Geo g, Geo gq, Phys P, MixedView M,
              const unsigned char* __restrict__ smap, const double* Uold, double* Unew,
              double coef, double* __restrict__ Rout, int sb, int nsk,
              unsigned int* __restrict__ err, Prim3Out On,
              unsigned long long* __restrict__ red_n) {
  extern __shared__ __align__(128) unsigned char smdyn[];
  unsigned char* smraw = aligned_smem(smdyn);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw);
  const SpecLayout L = spec_layout(NS);
  float* tiles = reinterpret_cast<float*>(smraw + BAR_BYTES);
  float* sG = tiles + NBUF * L.size;  // [2][TY][TX][NS]
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const Place pl = place_faces(g);
  const int i = pl.i, j = pl.j;
  const int kc0 = g.ng + (int)blockIdx.z * KZ3;
  const int kc1 = min(kc0 + KZ3, g.ngk - g.ng);
  const bool fi = i <= g.ngi - g.ng - 1;
  const bool fj = j <= g.ngj - g.ng - 1;
  const bool ci = tx >= 1 && i >= g.ng && i < g.ngi - g.ng;
  const bool cj = ty >= 1 && j >= g.ng && j < g.ngj - g.ng;
  const bool cell_col = ci && cj;
  const bool in_arr = i < g.ngi && j < g.ngj;
  const long long cq0 = (long long)i + gq.sy * j;
  const long long c0 = (long long)i + g.sy * j;
  const int s0 = 4 + sb;  // first Q field / state variable of this launch
  const float rd0 = P.rd_f[0], rd1 = P.rd_f[1], rd2 = P.rd_f[2];

  if (tid == 0) {
    prefetch_map(&maps.qs);
    prefetch_map(&maps.v2);
    for (int q = 0; q < NBUF; ++q) mbar_init(&bar[q], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int m) {
    const int buf = m % NBUF, k = kc0 + m;
    float* tb = tiles + buf * L.size;
    mbar_arrive_expect_tx(&bar[buf], L.bytes);
    tma_load_4d(tb + L.q, &maps.qs, &bar[buf], pl.x0, pl.y0, k, s0);
    tma_load_4d(tb + L.v, &maps.v2, &bar[buf], pl.x0, pl.y0, k, 0);
  };
  if (tid == 0) {
    issue(0);
    if (kc0 + 1 < kc1) issue(1);
  }

  // z-window of the own column: species and w at planes k-2 .. k+3 (the
  // new plane and the old state are loaded at the top of each iteration and
  // first used in its second half, after the x/y faces)
  float qz[NS][6], wz[6];
  const float* vz = M.vel + 2 * gq.sv;
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const long long o = cq0 + gq.sz * (kc0 - 3 + m);  // >= 0 (ng = 3)
#pragma unroll
    for (int s = 0; s < NS; ++s) qz[s][m] = (in_arr && s < nsk) ? M.Q[o + gq.sv * (s0 + s)] : 0.f;
    wz[m] = in_arr ? vz[o] : 0.f;
  }
  double uo[NS], um[4];
  float lS = -3.0e38f;

  float Gz[NS], Gx[NS], Gy[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) Gz[s] = Gx[s] = Gy[s] = 0.f;
  if (cell_col) {  // prologue: z face at kc0 - 1/2 from planes kc0-3 .. kc0+2
    const float uf = face_u(wz[1], wz[2], wz[3], wz[4]);
    const bool sm = HYB && smooth_at(smap, cq0 + gq.sz * (kc0 - 1), 2);
#pragma unroll
    for (int s = 0; s < NS; ++s) Gz[s] = uf * rd2 * rec5z<HYB>(qz[s], uf < 0.0f, sm);
  }

  bool ok = true;
  int k = kc0;
  for (; k < kc1; ++k) {
    const int n = k - kc0, b = n % NBUF;
    // window -> planes k-2 .. k+3 (plane k+3 <= kc1 + 2 < ngk); old state
#pragma unroll
    for (int m = 0; m < 5; ++m) {
#pragma unroll
      for (int s = 0; s < NS; ++s) qz[s][m] = qz[s][m + 1];
      wz[m] = wz[m + 1];
    }
    if (in_arr) {
      const long long o = cq0 + gq.sz * (k + 3);
#pragma unroll
      for (int s = 0; s < NS; ++s) qz[s][5] = s < nsk ? M.Q[o + gq.sv * (s0 + s)] : 0.f;
      wz[5] = vz[o];
    }
    if (cell_col && !Rout) {
      const long long c = c0 + g.sz * k;
#pragma unroll
      for (int s = 0; s < NS; ++s) uo[s] = s < nsk ? Uold[c + g.sv * (s0 + s)] : 0.0;
      if (EPI) {
#pragma unroll
        for (int w = 0; w < 4; ++w) um[w] = Unew[c + g.sv * w];
      }
    }
    ok = ok && mbar_wait(&bar[b], (uint32_t)((n / NBUF) & 1), err);
    const float* tb = tiles + b * L.size;
    const long long cqk = cq0 + gq.sz * k;
    float* sGk = sG + (n & 1) * (TY * TX * NS);
    if (ok && fi && cj) {  // x face at i+1/2
      const float* tv = tb + L.v + pl.own;
      const float uf = face_u(tv[-1], tv[0], tv[1], tv[2]);
      const bool neg = uf < 0.0f;
      const bool sm = HYB && smooth_at(smap, cqk, 0);
      const float sc = uf * rd0;
#pragma unroll
      for (int s = 0; s < NS; ++s)
        Gx[s] = sc * rec5<HYB>(tb + L.q + s * PL + pl.own, neg ? 3 : -2, neg ? -1 : 1, sm);
    }
    if (ok && fj && ci) {  // y face at j+1/2
      const float* tv = tb + L.v + PL + pl.own;
      const float uf = face_u(tv[-HX], tv[0], tv[HX], tv[2 * HX]);
      const bool neg = uf < 0.0f;
      const bool sm = HYB && smooth_at(smap, cqk, 1);
      const float sc = uf * rd1;
#pragma unroll
      for (int s = 0; s < NS; ++s)
        Gy[s] = sc * rec5<HYB>(tb + L.q + s * PL + pl.own, neg ? 3 * HX : -2 * HX,
                               neg ? -HX : HX, sm);
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) sGk[(ty * TX + tx) * NS + s] = Gy[s];
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    if (tid == 0 && k + 2 < kc1) {  // every thread is past plane k-1's buffer
      fence_proxy_async();
      issue(n + 2);
    }
    float Gzn[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) Gzn[s] = 0.f;
    if (cell_col) {  // z face at k+1/2
      const float uf = face_u(wz[1], wz[2], wz[3], wz[4]);
      const bool sm = HYB && smooth_at(smap, cqk, 2);
#pragma unroll
      for (int s = 0; s < NS; ++s) Gzn[s] = uf * rd2 * rec5z<HYB>(qz[s], uf < 0.0f, sm);
    }
    float R[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      const float gxl = __shfl_up_sync(0xffffffffu, Gx[s], 1);
      R[s] = 0.f;
      if (cell_col)
        R[s] = -((Gx[s] - gxl) + (Gy[s] - sGk[((ty - 1) * TX + tx) * NS + s]) + (Gzn[s] - Gz[s]));
    }
    if (cell_col) {
      const long long c = c0 + g.sz * k;
      double un[NS];
#pragma unroll
      for (int s = 0; s < NS; ++s) {
        if (s >= nsk) break;
        const long long a = c + g.sv * (s0 + s);
        if (Rout) {
          Rout[a] = f2d(R[s]);
        } else {
          un[s] = uo[s] + coef * f2d(R[s]);
          Unew[a] = un[s];
        }
      }
      if (EPI) {
        float sp;
        eos3<NS>(P, un, um, On, cqk, gq.sv, &sp);
        lS = fmaxf(lS, sp);
      }
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) Gz[s] = Gzn[s];
  }
  if (EPI) {  // interior maximum of |u| + c of U_new (maxWaveSpeed, src/ceq3d.hpp:25-63)
    lS = warp_maxf(lS);
    if ((tid & 31) == 0 && lS > -1e38f) atomicMax(&red_n[0], fst_key((double)lS));
  }
  if (!ok && tid == 0) {
    for (int m = k - kc0; m <= k - kc0 + 1 && kc0 + m < kc1; ++m)
      mbar_wait(&bar[m % NBUF], (uint32_t)((m / NBUF) & 1), err);
  }
}

// ---------------------------------------------------------------------------
// Momentum / energy face terms of one face (normal F), given its WENO
// fluxes in G: G[w] -= V[w]/d_F with V the viscous stress (and work) and the
// C-equation tensor term of the reference, from the 3x3 velocity gradient.
// ---------------------------------------------------------------------------
template <int F>
__device__ __forceinline__ void mom_face_terms(const Phys& P, const FaceCtx& fc,
                                               const float gr[3][3], float mu,
                                               const float uav[3], float r, float chat,
                                               const float cn[3], float* G) {
  float V[4] = {0.f, 0.f, 0.f, 0.f};
  if (P.visc) {
    const float div = gr[0][0] + gr[1][1] + gr[2][2];
    float e = 0.f;
#pragma unroll
    for (int w = 0; w < 3; ++w) {
      const float Tw = (w == F) ? (2.0f / 3.0f) * mu * (3.0f * gr[F][F] - div)
                                : mu * (gr[F][w] + gr[w][F]);
      e += uav[w] * Tw;
      V[w] += Tw;
    }
    V[3] = e;
  }
  if (P.ceq) {
    const float cmag = 1.0e-6f + cn[0] * cn[0] + cn[1] * cn[1] + cn[2] * cn[2];
    const float rc = __fdividef(1.0f, cmag);
    const float arc = fc.alpha * r * chat;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float base = arc * ((F == d ? 1.0f : 0.0f) - cn[F] * cn[d] * rc);
#pragma unroll
      for (int w = 0; w < 3; ++w) V[w] += base * gr[d][w];
    }
  }
#pragma unroll
  for (int w = 0; w < 4; ++w) G[w] -= V[w] * fc.rd[F];
}

// Velocity gradient on the face with normal F owned by the thread's cell:
// gr[d][w] = d u_w / d x_d, from the velocity planes k-1 (pm), k (p0) and
// k+1 (pp), each pointing at the thread's cell of field u.
template <int F>
__device__ __forceinline__ void face_grad(const float* pm, const float* p0, const float* pp,
                                          const FaceCtx& fc, float gr[3][3], float uav[3]) {
  constexpr int fk = F == 2, fr = F == 1, fcx = F == 0;
  auto U = [&](int w, int dk, int dr, int dc) -> float {
    const float* p = dk < 0 ? pm : (dk > 0 ? pp : p0);
    return p[w * PL + dr * HX + dc];
  };
#pragma unroll
  for (int w = 0; w < 3; ++w) {
    uav[w] = 0.5f * (U(w, fk, fr, fcx) + U(w, 0, 0, 0));
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (d == F) {
        gr[d][w] = (U(w, fk, fr, fcx) - U(w, 0, 0, 0)) * fc.rd[d];
      } else {
        const int tk = d == 2, tr = d == 1, tc = d == 0;
        gr[d][w] = ((U(w, fk + tk, fr + tr, fcx + tc) + U(w, tk, tr, tc)) -
                    (U(w, fk - tk, fr - tr, fcx - tc) + U(w, -tk, -tr, -tc))) *
                   fc.r4d[d];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// k_mmom3d: face terms of the momenta and energy, added to the cell terms
// k_mcell3d wrote: U_new += coef * R_face (or R += R_face)
// ---------------------------------------------------------------------------
template <bool HYB>
__global__ void __launch_bounds__(TX * TY, 2)
    k_mmom3d(const __grid_constant__ Mixed3DMaps maps, Geo g, Geo gq, Phys P, MixedView M,
             const unsigned long long* __restrict__ red, const unsigned char* __restrict__ smap,
             double* Unew, double coef, double* __restrict__ Rout,
             unsigned int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smdyn[];
  unsigned char* smraw = aligned_smem(smdyn);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw);  // [0..2] tiles, [3..7] velocity ring
  const bool visc = P.visc != 0, ceq = P.ceq != 0;
  const MomLayout L = mom_layout(visc, ceq);
  float* tiles = reinterpret_cast<float*>(smraw + BAR_BYTES);
  float* ring = tiles + NBUF * L.tsize;
  float* sG = ring + NRING * L.rsize;  // [2][TY][TX][4]
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const Place pl = place_faces(g);
  const int i = pl.i, j = pl.j;
  const int kc0 = g.ng + (int)blockIdx.z * KZ3;
  const int kc1 = min(kc0 + KZ3, g.ngk - g.ng);
  const bool fi = i <= g.ngi - g.ng - 1;
  const bool fj = j <= g.ngj - g.ng - 1;
  const bool ci = tx >= 1 && i >= g.ng && i < g.ngi - g.ng;
  const bool cj = ty >= 1 && j >= g.ng && j < g.ngj - g.ng;
  const bool cell_col = ci && cj;
  const bool in_arr = i < g.ngi && j < g.ngj;
  const long long cq0 = (long long)i + gq.sy * j;
  const long long c0 = (long long)i + g.sy * j;
  double* Ub = Rout ? Rout : Unew;  // what k_mcell3d wrote
  const double cf = Rout ? 1.0 : coef;
  float maxS;
  const FaceCtx fc = make_ctx(P, red, &maxS);

  if (tid == 0) {
    prefetch_map(&maps.q4);
    prefetch_map(&maps.v3);
    for (int q = 0; q < NBUF + NRING; ++q) mbar_init(&bar[q], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue_tile = [&](int m) {  // plane kc0 + m into buffer m % NBUF
    const int buf = m % NBUF, k = kc0 + m;
    float* tb = tiles + buf * L.tsize;
    mbar_arrive_expect_tx(&bar[buf], L.tbytes);
    tma_load_4d(tb + L.q, &maps.q4, &bar[buf], pl.x0, pl.y0, k, 0);
    if (visc) tma_load_4d(tb + L.mu, &maps.mu, &bar[buf], pl.x0, pl.y0, k, 0);
    if (ceq) {
      tma_load_4d(tb + L.rho, &maps.rho, &bar[buf], pl.x0, pl.y0, k, 0);
      tma_load_4d(tb + L.c, &maps.c4, &bar[buf], pl.x0, pl.y0, k, 1);
    }
  };
  auto wait_tile = [&](int m) {
    return mbar_wait(&bar[m % NBUF], (uint32_t)((m / NBUF) & 1), err);
  };
  // velocity plane p (>= kc0-2) lives in ring slot (p - kc0 + 2) % NRING
  auto issue_vel = [&](int p) {
    const int r = p - kc0 + 2, s = r % NRING;
    mbar_arrive_expect_tx(&bar[NBUF + s], L.rbytes);
    tma_load_4d(ring + s * L.rsize, &maps.v3, &bar[NBUF + s], pl.x0, pl.y0, p, 0);
  };
  auto wait_vel = [&](int p) {
    const int r = p - kc0 + 2;
    return mbar_wait(&bar[NBUF + r % NRING], (uint32_t)((r / NRING) & 1), err);
  };
  auto vel_at = [&](int p) -> const float* {
    return ring + ((p - kc0 + 2) % NRING) * L.rsize + pl.own;
  };
  if (tid == 0) {
    for (int p = kc0 - 2; p <= kc0 + 2; ++p) issue_vel(p);  // planes <= kc1 + 1 < ngk
    issue_tile(0);
    issue_tile(1);  // plane kc0 + 1 <= kc1 <= ngk - 3
  }

  // z-window of the own column: Q0..3 at planes k-2 .. k+3 (new plane and
  // the U_new base loaded at the top of each iteration)
  float qz[4][6];
#pragma unroll
  for (int m = 0; m < 6; ++m)
#pragma unroll
    for (int v = 0; v < 4; ++v)
      qz[v][m] = in_arr ? M.Q[cq0 + gq.sv * v + gq.sz * (kc0 - 3 + m)] : 0.f;
  double ub[4] = {0.0, 0.0, 0.0, 0.0};

  // face averages on the z face between planes ka and ka+1 of the own column
  auto zface_scalars = [&](float a_mu, float b_mu, float a_r, float b_r, const float* a_c,
                           const float* b_c, float& mu, float& r, float& chat, float cn[3]) {
    mu = 0.5f * (a_mu + b_mu);
    r = 0.5f * (a_r + b_r);
    chat = 0.5f * (a_c[0] + b_c[0]);
#pragma unroll
    for (int q = 0; q < 3; ++q) cn[q] = 0.5f * (a_c[1 + q] + b_c[1 + q]);
  };

  float Gz[4] = {0.f, 0.f, 0.f, 0.f};
  float Gx[4] = {0.f, 0.f, 0.f, 0.f}, Gy[4] = {0.f, 0.f, 0.f, 0.f};
  bool ok = true;
  for (int p = kc0 - 2; p <= kc0 + 1; ++p) ok = wait_vel(p) && ok;
  if (cell_col && ok) {  // prologue: z face at kc0 - 1/2
    const int ka = kc0 - 1;
    const float *um = vel_at(ka - 1), *u0 = vel_at(ka), *u1 = vel_at(ka + 1), *u2 = vel_at(ka + 2);
    const float uf = face_u(um[2 * PL], u0[2 * PL], u1[2 * PL], u2[2 * PL]);
    const bool neg = uf < 0.0f;
    const long long ca = cq0 + gq.sz * ka, cb = ca + gq.sz;
    const bool sm = HYB && smooth_at(smap, ca, 2);
#pragma unroll
    for (int v = 0; v < 4; ++v) Gz[v] = uf * fc.rd[2] * rec5z<HYB>(qz[v], neg, sm);
    if (visc || ceq) {
      float gr[3][3], uav[3], mu = 0.f, r = 0.f, chat = 0.f, cn[3] = {0.f, 0.f, 0.f};
      face_grad<2>(um, u0, u1, fc, gr, uav);
      float ac[4] = {0.f, 0.f, 0.f, 0.f}, bc[4] = {0.f, 0.f, 0.f, 0.f};
      if (ceq)
        for (int q = 0; q < 4; ++q) {
          ac[q] = M.C[ca + gq.sv * (1 + q)];
          bc[q] = M.C[cb + gq.sv * (1 + q)];
        }
      zface_scalars(visc ? M.mu[ca] : 0.f, visc ? M.mu[cb] : 0.f, ceq ? M.rho[ca] : 0.f,
                    ceq ? M.rho[cb] : 0.f, ac, bc, mu, r, chat, cn);
      mom_face_terms<2>(P, fc, gr, mu, uav, r, chat, cn, Gz);
    }
  }

  int k = kc0;
  for (; k < kc1; ++k) {
    const int n = k - kc0;
#pragma unroll
    for (int m = 0; m < 5; ++m)
#pragma unroll
      for (int v = 0; v < 4; ++v) qz[v][m] = qz[v][m + 1];
    if (in_arr) {
      const long long o = cq0 + gq.sz * (k + 3);  // plane k+3 <= kc1 + 2 < ngk
#pragma unroll
      for (int v = 0; v < 4; ++v) qz[v][5] = M.Q[o + gq.sv * v];
    }
    if (cell_col)
#pragma unroll
      for (int w = 0; w < 4; ++w) ub[w] = Ub[c0 + g.sz * k + g.sv * w];
    ok = ok && wait_tile(n);
    const float* tb = tiles + (n % NBUF) * L.tsize;
    const float *um = vel_at(k - 1), *u0 = vel_at(k), *u1 = vel_at(k + 1);
    const long long cqk = cq0 + gq.sz * k;
    float* sGk = sG + (n & 1) * (TY * TX * 4);
    if (ok && fi && cj) {  // x face at i+1/2
      const float uf = face_u(u0[-1], u0[0], u0[1], u0[2]);
      const bool neg = uf < 0.0f;
      const bool sm = HYB && smooth_at(smap, cqk, 0);
      const float sc = uf * fc.rd[0];
#pragma unroll
      for (int v = 0; v < 4; ++v)
        Gx[v] = sc * rec5<HYB>(tb + L.q + v * PL + pl.own, neg ? 3 : -2, neg ? -1 : 1, sm);
      if (visc || ceq) {
        float gr[3][3], uav[3], mu = 0.f, r = 0.f, chat = 0.f, cn[3] = {0.f, 0.f, 0.f};
        face_grad<0>(um, u0, u1, fc, gr, uav);
        const int o = pl.own;
        if (visc) mu = 0.5f * (tb[L.mu + o] + tb[L.mu + o + 1]);
        if (ceq) {
          r = 0.5f * (tb[L.rho + o] + tb[L.rho + o + 1]);
          chat = 0.5f * (tb[L.c + o] + tb[L.c + o + 1]);
#pragma unroll
          for (int q = 0; q < 3; ++q)
            cn[q] = 0.5f * (tb[L.c + (1 + q) * PL + o] + tb[L.c + (1 + q) * PL + o + 1]);
        }
        mom_face_terms<0>(P, fc, gr, mu, uav, r, chat, cn, Gx);
      }
    }
    if (ok && fj && ci) {  // y face at j+1/2
      const float* w0 = u0 + PL;
      const float uf = face_u(w0[-HX], w0[0], w0[HX], w0[2 * HX]);
      const bool neg = uf < 0.0f;
      const bool sm = HYB && smooth_at(smap, cqk, 1);
      const float sc = uf * fc.rd[1];
#pragma unroll
      for (int v = 0; v < 4; ++v)
        Gy[v] = sc * rec5<HYB>(tb + L.q + v * PL + pl.own, neg ? 3 * HX : -2 * HX, neg ? -HX : HX,
                               sm);
      if (visc || ceq) {
        float gr[3][3], uav[3], mu = 0.f, r = 0.f, chat = 0.f, cn[3] = {0.f, 0.f, 0.f};
        face_grad<1>(um, u0, u1, fc, gr, uav);
        const int o = pl.own;
        if (visc) mu = 0.5f * (tb[L.mu + o] + tb[L.mu + o + HX]);
        if (ceq) {
          r = 0.5f * (tb[L.rho + o] + tb[L.rho + o + HX]);
          chat = 0.5f * (tb[L.c + o] + tb[L.c + o + HX]);
#pragma unroll
          for (int q = 0; q < 3; ++q)
            cn[q] = 0.5f * (tb[L.c + (1 + q) * PL + o] + tb[L.c + (1 + q) * PL + o + HX]);
        }
        mom_face_terms<1>(P, fc, gr, mu, uav, r, chat, cn, Gy);
      }
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) sGk[(ty * TX + tx) * 4 + v] = Gy[v];
    ok = ok && wait_vel(k + 2);
    ok = ok && wait_tile(n + 1);
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    if (tid == 0) {  // every thread is past plane k-1's tile and plane k-2's velocities
      fence_proxy_async();
      if (k + 2 <= kc1) issue_tile(n + 2);
      if (k + 3 <= kc1 + 1) issue_vel(k + 3);
    }
    float Gzn[4] = {0.f, 0.f, 0.f, 0.f};
    if (cell_col) {  // z face at k+1/2: own column, planes k and k+1 (next tile)
      const float* u2 = vel_at(k + 2);
      const float uf = face_u(um[2 * PL], u0[2 * PL], u1[2 * PL], u2[2 * PL]);
      const bool neg = uf < 0.0f;
      const bool sm = HYB && smooth_at(smap, cqk, 2);
#pragma unroll
      for (int v = 0; v < 4; ++v) Gzn[v] = uf * fc.rd[2] * rec5z<HYB>(qz[v], neg, sm);
      if (visc || ceq) {
        const float* tn = tiles + ((n + 1) % NBUF) * L.tsize;
        float gr[3][3], uav[3], mu = 0.f, r = 0.f, chat = 0.f, cn[3] = {0.f, 0.f, 0.f};
        face_grad<2>(um, u0, u1, fc, gr, uav);
        const int o = pl.own;
        float ac[4], bc[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          ac[q] = tb[L.c + q * PL + o];
          bc[q] = tn[L.c + q * PL + o];
        }
        zface_scalars(tb[L.mu + o], tn[L.mu + o], tb[L.rho + o], tn[L.rho + o], ac, bc, mu, r,
                      chat, cn);
        mom_face_terms<2>(P, fc, gr, mu, uav, r, chat, cn, Gzn);
      }
    }
    float R[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const float gxl = __shfl_up_sync(0xffffffffu, Gx[v], 1);
      R[v] = 0.f;
      if (cell_col)
        R[v] = -((Gx[v] - gxl) + (Gy[v] - sGk[((ty - 1) * TX + tx) * 4 + v]) + (Gzn[v] - Gz[v]));
    }
    if (cell_col) {
      const long long c = c0 + g.sz * k;
#pragma unroll
      for (int w = 0; w < 4; ++w) Ub[c + g.sv * w] = ub[w] + cf * f2d(R[w]);
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) Gz[v] = Gzn[v];
  }
  if (!ok && tid == 0) {
    // a wait ran out: let the copies in flight land (bounded)
    const int n = k - kc0;
    for (int m = n; m <= n + 1 && kc0 + m <= kc1; ++m) wait_tile(m);
    for (int p = k + 1; p <= k + 2 && p <= kc1 + 1; ++p) wait_vel(p);
  }
}

inline unsigned cdiv3(long long a, int b) { return (unsigned)((a + b - 1) / b); }

size_t spec_smem(int nsc) {
  return ALIGN_SLACK + BAR_BYTES +
         sizeof(float) * (NBUF * (size_t)spec_layout(nsc).size + 2 * (size_t)TY * TX * nsc);
}
size_t mom_smem(bool visc, bool ceq) {
  const MomLayout L = mom_layout(visc, ceq);
  return ALIGN_SLACK + BAR_BYTES +
         sizeof(float) * (NBUF * (size_t)L.tsize + NRING * (size_t)L.rsize + 2 * (size_t)TY * TX * 4);
}
size_t cell_smem() {
  return ALIGN_SLACK + BAR_BYTES + sizeof(float) * NBUF * (size_t)cell_layout().size;
}
size_t ceq_smem() {
  return ALIGN_SLACK + BAR_BYTES + sizeof(float) * NBUF * (size_t)ceq_layout().size;
}

template <int NS, bool HYB>
int launch_spec(const Geo& g, const Phys& P, const MixedBufs& b, const MixedView& M,
                const unsigned char* smooth, const double* Uold, double* Unew, double coef,
                double* Rout, cudaStream_t st, bool fused) {
  const dim3 grd(cdiv3(g.nci, TX - 1), cdiv3(g.ncj, TY - 1), cdiv3(g.nck, KZ3));
  const size_t sm = spec_smem(NS);
  if (fused) {  // one launch over all species, with the equation-of-state epilogue
    const PrimSet& A = b.alt;
    const Prim3Out On{A.Q, A.rho32, A.vel32, A.p32, P.visc ? A.mu32 : nullptr,
                      P.ceq ? A.nrg : nullptr, nullptr, P.ceq ? A.plo : nullptr, A.rho64};
    cudaFuncSetAttribute(k_mspec3d<NS, HYB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    k_mspec3d<NS, HYB, true><<<grd, dim3(TX, TY), sm, st>>>(
        *b.maps3d, g, b.gq, P, M, smooth, Uold, Unew, coef, Rout, 0, g.ns, b.dev_err, On, A.red);
    return 1;
  }
  cudaFuncSetAttribute(k_mspec3d<NS, HYB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sm);
  int n = 0;
  for (int sb = 0; sb < g.ns; sb += NS) {
    const int nsk = g.ns - sb < NS ? g.ns - sb : NS;
    k_mspec3d<NS, HYB, false><<<grd, dim3(TX, TY), sm, st>>>(*b.maps3d, g, b.gq, P, M, smooth,
                                                             Uold, Unew, coef, Rout, sb, nsk,
                                                             b.dev_err, Prim3Out{}, nullptr);
    ++n;
  }
  return n;
}

template <bool HYB>
int launch_spec_any(const Geo& g, const Phys& P, const MixedBufs& b, const MixedView& M,
                    const unsigned char* smooth, const double* Uold, double* Unew, double coef,
                    double* Rout, cudaStream_t st, bool fused) {
  switch (b.maps3d->nsc) {
    case 1: return launch_spec<1, HYB>(g, P, b, M, smooth, Uold, Unew, coef, Rout, st, fused);
    case 2: return launch_spec<2, HYB>(g, P, b, M, smooth, Uold, Unew, coef, Rout, st, fused);
    case 3: return launch_spec<3, HYB>(g, P, b, M, smooth, Uold, Unew, coef, Rout, st, fused);
    case 4: return launch_spec<4, HYB>(g, P, b, M, smooth, Uold, Unew, coef, Rout, st, fused);
    default: return launch_spec<5, HYB>(g, P, b, M, smooth, Uold, Unew, coef, Rout, st, fused);
  }
}

template <bool HYB>
void launch_mom(const Geo& g, const Phys& P, const MixedBufs& b, const MixedView& M,
                const unsigned char* smooth, double* Unew, double coef, double* Rout,
                cudaStream_t st) {
  const dim3 grd(cdiv3(g.nci, TX - 1), cdiv3(g.ncj, TY - 1), cdiv3(g.nck, KZ3));
  const size_t sm = mom_smem(P.visc != 0, P.ceq != 0);
  cudaFuncSetAttribute(k_mmom3d<HYB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_mmom3d<HYB><<<grd, dim3(TX, TY), sm, st>>>(*b.maps3d, g, b.gq, P, M, b.red, smooth, Unew,
                                              coef, Rout, b.dev_err);
}

void launch_cell(const Geo& g, const Phys& P, const MixedBufs& b, const MixedView& M,
                 const double* Uold, double* Unew, double coef, double* Rout, cudaStream_t st) {
  const dim3 grd(cdiv3(g.nci, TX), cdiv3(g.ncj, TY), cdiv3(g.nck, KZ3));
  const size_t sm = cell_smem();
  cudaFuncSetAttribute(k_mcell3d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_mcell3d<<<grd, dim3(TX, TY), sm, st>>>(*b.maps3d, g, b.gq, P, M, Uold, Unew, coef, Rout,
                                          b.dev_err);
}

void launch_ceq(const Geo& g, const Phys& P, const MixedBufs& b, const MixedView& M,
                const double* Uold, double* Unew, double coef, double* Rout, cudaStream_t st,
                bool fused) {
  const dim3 grd(cdiv3(g.nci, TX), cdiv3(g.ncj, TY), cdiv3(g.nck, KZ3));
  const size_t sm = ceq_smem();
  cudaFuncSetAttribute(k_mceq3d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_mceq3d<<<grd, dim3(TX, TY), sm, st>>>(*b.maps3d, g, b.gq, P, M, b.red, Uold, Unew, coef,
                                         Rout, b.dev_err, fused ? b.alt.C : nullptr,
                                         fused ? b.alt.red : nullptr);
}

// species per k_mspec3d launch: all of them up to 5, else chunks of 4
int species_chunk(int ns) { return ns <= 5 ? ns : 4; }

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 4D map (x, y, z, field) over a primitive array of nf fields, box
// (HX, HY, 1, box_f); 4- or 8-byte elements.
bool make_map(CUtensorMap* m, const Geo& g, const Geo& gq, const void* base, int nf, int box_f,
              bool f64, std::string* why) {
  auto fn = encode_fn();
  if (!fn) {
    if (why) *why = "cuTensorMapEncodeTiled is not available from the driver";
    return false;
  }
  const size_t es = f64 ? 8 : 4;
  cuuint64_t dims[4] = {(cuuint64_t)g.ngi, (cuuint64_t)g.ngj, (cuuint64_t)g.ngk, (cuuint64_t)nf};
  cuuint64_t strides[3] = {(cuuint64_t)(gq.sy * es), (cuuint64_t)(gq.sz * es),
                           (cuuint64_t)(gq.sv * es)};
  cuuint32_t box[4] = {(cuuint32_t)HX, (cuuint32_t)HY, 1u, (cuuint32_t)box_f};
  cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
  CUresult r = fn(m, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                  const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    if (why) *why = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")";
    return false;
  }
  return true;
}

}  // namespace

Geo fst_prim_geo(const Geo& g) {
  Geo q = g;
  if (g.ndim == 3) {
    q.sy = (g.ngi + 3) & ~3;  // rows of whole 16-byte groups
    q.sz = q.sy * g.ngj;
    q.sv = q.sz * g.ngk;
  }
  return q;
}

namespace {
// tensor maps over one set of primitive arrays
int build_maps(const Geo& g, const Geo& gq, const float* Q, const float* vel32, const float* p32,
               const float* rho32, const float* nrg, const float* mu32, const float* C,
               const float* plo, Mixed3DMaps** out, std::string* why) {
  Mixed3DMaps* m = new (std::nothrow) Mixed3DMaps();
  if (!m) return FST_ERR_OOM;
  m->nsc = species_chunk(g.ns);
  bool ok = make_map(&m->qs, g, gq, Q, g.nv, m->nsc, false, why) &&
            make_map(&m->q4, g, gq, Q, g.nv, 4, false, why) &&
            make_map(&m->v2, g, gq, vel32, 3, 2, false, why) &&
            make_map(&m->v3, g, gq, vel32, 3, 3, false, why) &&
            make_map(&m->p, g, gq, p32, 2, 2, false, why);
  if (ok && rho32) ok = make_map(&m->rho, g, gq, rho32, 1, 1, false, why);
  if (ok && nrg) ok = make_map(&m->nrg, g, gq, nrg, 1, 1, false, why);
  if (ok && mu32) ok = make_map(&m->mu, g, gq, mu32, 1, 1, false, why);
  if (ok && C) ok = make_map(&m->c5, g, gq, C, 5, 5, false, why) &&
                    make_map(&m->c4, g, gq, C, 5, 4, false, why);
  if (ok && plo) ok = make_map(&m->lo4, g, gq, plo, 5, 4, false, why);
  if (!ok) {
    delete m;
    return FST_ERR_CUDA;
  }
  *out = m;
  return FST_OK;
}
}  // namespace

int fst_mixed3d_prepare(const Geo& g, MixedBufs& b, std::string* why) {
  if (g.ndim != 3) return FST_OK;
  if (g.ng != 3) {
    if (why) *why = "the 3D mixed kernels need ng = 3";
    return FST_ERR_UNSUPPORTED;
  }
  int rc = build_maps(g, b.gq, b.Q, b.vel32, b.p32, b.rho32, b.nrg, b.mu32, b.C, b.plo,
                      &b.maps3d, why);
  if (rc == FST_OK && b.fused) {
    const PrimSet& A = b.alt;
    rc = build_maps(g, b.gq, A.Q, A.vel32, A.p32, A.rho32, A.nrg, A.mu32, A.C, A.plo,
                    &b.alt.maps3d, why);
  }
  return rc;
}

void fst_mixed3d_release(MixedBufs& b) {
  delete b.maps3d;
  b.maps3d = nullptr;
  delete b.alt.maps3d;
  b.alt.maps3d = nullptr;
}

namespace {
// fst_rk_step_get_state: once the kernels enqueued so far have run, copy
// variables [v0, v0 + nvar) of U to the host on the side stream
void download_group(const Geo& g, MixedDownload* dl, int bit, int slot, const double* U, int v0,
                    int nvar, cudaStream_t st) {
  if (!dl || nvar <= 0) return;
  cudaEventRecord(dl->ev[slot], st);
  cudaStreamWaitEvent(dl->side, dl->ev[slot], 0);
  const size_t off = (size_t)g.sv * v0;
  cudaMemcpyAsync(dl->host + off, U + off, sizeof(double) * g.sv * nvar, cudaMemcpyDeviceToHost,
                  dl->side);
  dl->issued |= bit;
}
}  // namespace

int fst_mixed3d_rhs(const Geo& g, const Phys& P, const MixedBufs& b, const MixedView& M,
                    const unsigned char* smooth, const double* Uold, double* Unew, double coef,
                    double* Rout, cudaStream_t st, Prof* prof, bool hybrid, bool fused) {
  int n = 0;
  // a final stage that downloads as it goes (never with a bare RHS)
  MixedDownload* dl = Rout ? nullptr : b.dl;
  // cell terms before the face terms: k_mmom3d adds its face terms to what
  // k_mcell3d wrote (on a generalized grid, the metric pressure gradient)
  if (b.metf) {
    FST_LAUNCH(prof, "gen_cell", st, n,
               fst_mixedgen_cell(g, b.gq, M, b.metf, Uold, Unew, coef, Rout, st));
  } else {
    // the C variables first (k_mceq3d and k_mcell3d write disjoint
    // variables): a download of U_new starts on them soonest
    if (P.ceq) {
      FST_LAUNCH(prof, "mceq3d", st, n,
                 launch_ceq(g, P, b, M, Uold, Unew, coef, Rout, st, fused));
      download_group(g, dl, FST_DL_CEQ, 0, Unew, g.nv, 5, st);  // C is complete
    }
    FST_LAUNCH(prof, "mcell3d", st, n, launch_cell(g, P, b, M, Uold, Unew, coef, Rout, st));
  }
  // fused stages: the species kernel runs last, after the momenta and energy
  // of U_new are complete, and evaluates the next stage's primitives
  auto spec = [&]() {
    const char* nm = fused ? (hybrid ? "mspec3d_hybrid_eos" : "mspec3d_eos")
                           : (hybrid ? "mspec3d_hybrid" : "mspec3d");
    if (hybrid)
      FST_LAUNCH(prof, nm, st, n,
                 n += launch_spec_any<true>(g, P, b, M, smooth, Uold, Unew, coef, Rout, st,
                                            fused) - 1);
    else
      FST_LAUNCH(prof, nm, st, n,
                 n += launch_spec_any<false>(g, P, b, M, nullptr, Uold, Unew, coef, Rout, st,
                                             fused) - 1);
    download_group(g, dl, FST_DL_SPECIES, 1, Unew, 4, g.ns, st);  // species complete
  };
  if (!fused) spec();
  if (hybrid)
    FST_LAUNCH(prof, "mmom3d_hybrid", st, n,
               launch_mom<true>(g, P, b, M, smooth, Unew, coef, Rout, st));
  else
    FST_LAUNCH(prof, "mmom3d", st, n, launch_mom<false>(g, P, b, M, nullptr, Unew, coef, Rout, st));
  download_group(g, dl, FST_DL_MOMENTA, 2, Unew, 0, 4, st);  // momenta and energy complete
  if (fused) spec();
  return n;
}
