// fst_mixed.cu — mixed-precision right-hand side + RK stage (FST_MODE_MIXED)
// and the fused kernel shared with the learned-hybrid variant
// (FST_MODE_HYBRID) for sm_103a.
//
// Precision split:
//   FP64  the conserved state, the RK stage combine, the equation of state
//         (rho, mass fractions, gamma, p = (gamma-1)*(E - KE): the low-Mach
//         cancellation), the stored pressure and its 4th-order gradient,
//         E + p, and the buoyancy source
//   FP32  velocities, WENO5 reconstruction and fluxes, viscous stress,
//         C-equation terms, the wave-speed and C_hat maxima
//
// Per stage: k_mprim over all cells (FP64 state -> FP32 primitives + FP64
// p, and the C-equation maxima maxS, maxCh by warp max + atomicMax), then
// the fused right-hand side + RK stage: in 3D the two TMA-fed kernels of
// fst_mixed3d.cu, in 2D k_mrhs2d below (a 32x8 tile of columns; each thread
// computes the faces at i+1/2 and j+1/2 once, the left x face by shuffle,
// the lower y face through shared memory; every face carries nv FP32
// values G_v = F_v - V_v/d: the WENO flux, and for the momenta and energy
// the viscous and C-equation face terms).  Face and stress arrays never go
// to HBM.  Kernels are instantiated per variable count so every
// per-variable array lives in registers.  The equations, quirks included,
// are the reference's (src/flux.hpp, src/viscosity.hpp, src/ceq.hpp,
// src/ceq3d.hpp, src/presgrad.hpp, src/buoyancy.hpp); only the arithmetic
// precision differs.  The error against the FP64 oracle is measured by
// tests/test_gpu_mixed.py.
#include <cstdlib>
#include <utility>

#include "fst_mixed_dev.cuh"

namespace {
using namespace fstm;

template <int NDIM>
__global__ void __launch_bounds__(256) k_mprim(Geo g, Geo gq, Phys P, const double* __restrict__ U,
                                               float* __restrict__ Q, float* __restrict__ rho,
                                               double* __restrict__ rho64,
                                               float* __restrict__ vel, double* __restrict__ pr,
                                               float* __restrict__ pp,
                                               float* __restrict__ mu, float* __restrict__ nrg,
                                               float* __restrict__ Cc, float* __restrict__ T,
                                               float* __restrict__ lo,
                                               unsigned long long* __restrict__ red) {
  // grid: x runs over the cells of one (i, j) plane in storage order, in
  // blocks of 256 across row ends (streaming, no idle threads), z = k
  const int t = blockIdx.x * 256 + threadIdx.x;
  const int j = t / g.ngi, i = t - j * g.ngi;
  float lS = -3.0e38f, lC = -3.0e38f;
  if (j < g.ngj)
    mprim_cell<NDIM>(g, gq, P, U, Q, rho, rho64, vel, pr, pp, mu, nrg, Cc, T, lo, red != nullptr, i, j,
                     blockIdx.z, lS, lC);
  if (red) {
    lS = warp_maxf(lS);
    lC = warp_maxf(lC);
    if ((threadIdx.x & 31) == 0 && lS > -1e38f) {
      atomicMax(&red[0], fst_key((double)lS));
      atomicMax(&red[1], fst_key((double)lC));
    }
  }
}

// 3D: the FP64-free equation of state of mprim3_cell, same grid as k_mprim
template <int NS>
__global__ void __launch_bounds__(256) k_mprim3(Geo g, Geo gq, Phys P,
                                                const double* __restrict__ U, Prim3Out O,
                                                unsigned long long* __restrict__ red) {
  const int t = blockIdx.x * 256 + threadIdx.x;
  const int j = t / g.ngi, i = t - j * g.ngi;
  float lS = -3.0e38f, lC = -3.0e38f;
  if (j < g.ngj) mprim3_cell<NS>(g, gq, P, U, O, red != nullptr, i, j, blockIdx.z, lS, lC);
  if (red) {
    lS = warp_maxf(lS);
    lC = warp_maxf(lC);
    if ((threadIdx.x & 31) == 0 && lS > -1e38f) {
      atomicMax(&red[0], fst_key((double)lS));
      atomicMax(&red[1], fst_key((double)lC));
    }
  }
}

// The ghost cells of the 3D primitive pass (fst_shell_cell order), one
// thread per cell.  Fused stages compute the interior in the previous
// stage's last kernel and only these after the boundary fill.
template <int NS>
__global__ void __launch_bounds__(256) k_mprim3_shell(Geo g, Geo gq, Phys P,
                                                      const double* __restrict__ U, Prim3Out O) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= fst_shell_count(g)) return;
  int i, j, k;
  fst_shell_cell(g, t, i, j, k);
  float lS = 0.f, lC = 0.f;
  mprim3_cell<NS>(g, gq, P, U, O, false, i, j, k, lS, lC);
}

// Fused upload: one thread per cell in storage order (as k_mprim3).  Every
// state value comes from host memory over the host link and goes to U; the
// interior cells also take mprim3_vals into the current primitive set.
template <int NS>
__global__ void __launch_bounds__(256) k_mupload3(Geo g, Geo gq, Phys P,
                                                  const double* __restrict__ Uh,
                                                  double* __restrict__ U, Prim3Out O,
                                                  unsigned long long* __restrict__ red) {
  const int t = blockIdx.x * 256 + threadIdx.x;
  const int j = t / g.ngi, i = t - j * g.ngi, k = blockIdx.z;
  float lS = -3.0e38f, lC = -3.0e38f;
  if (j < g.ngj) {
    const long long sv = g.sv;
    const long long c = (long long)i + g.sy * j + g.sz * k;
    const bool ceq = g.nvt > g.nv;
    double us[NS], um[4], uc[5];
#pragma unroll
    for (int s = 0; s < NS; ++s) us[s] = Uh[c + sv * (4 + s)];
#pragma unroll
    for (int d = 0; d < 4; ++d) um[d] = Uh[c + sv * d];
    if (ceq) {
#pragma unroll
      for (int n = 0; n < 5; ++n) uc[n] = Uh[c + sv * (g.nv + n)];
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) U[c + sv * (4 + s)] = us[s];
#pragma unroll
    for (int d = 0; d < 4; ++d) U[c + sv * d] = um[d];
    if (ceq) {
#pragma unroll
      for (int n = 0; n < 5; ++n) U[c + sv * (g.nv + n)] = uc[n];
    }
    const bool in = i >= g.ng && i < g.ngi - g.ng && j >= g.ng && j < g.ngj - g.ng &&
                    k >= g.ng && k < g.ngk - g.ng;
    if (in)
      mprim3_vals<NS>(g, P, us, um, uc, O, (long long)i + gq.sy * j + gq.sz * k, gq.sv,
                      red != nullptr, i, j, k, lS, lC);
  }
  if (red) {
    lS = warp_maxf(lS);
    lC = warp_maxf(lC);
    if ((threadIdx.x & 31) == 0 && lS > -1e38f) {
      atomicMax(&red[0], fst_key((double)lS));
      atomicMax(&red[1], fst_key((double)lC));
    }
  }
}

template <int NV, bool HYB>
__global__ void __launch_bounds__(TX * TY) k_mrhs2d(Geo g, Phys P, MixedView M,
                                                    const unsigned long long* __restrict__ red,
                                                    const unsigned char* __restrict__ smap,
                                                    const double* Uold, double* Unew, double coef,
                                                    double* __restrict__ Rout) {
  __shared__ float sG[TY][TX][NV];
  rhs2d_tile<NV, HYB, TY>(g, P, M, red, smap, Uold, Unew, coef, Rout, blockIdx.x, blockIdx.y, sG);
}

// ghost cells of the stage-1 buffer: U1 = U + (0.5*dt)*0 (src/rk.cpp:42-50).
// One thread per (ghost cell, variable), the cells in fst_shell_cell order.
__global__ void __launch_bounds__(256) k_mghost(Geo g, long long nshell,
                                                const double* __restrict__ Uold,
                                                double* __restrict__ Unew) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= nshell * g.nvt) return;
  const int v = (int)(t / nshell);
  int i, j, k;
  fst_shell_cell(g, t - (long long)v * nshell, i, j, k);
  const long long c = (long long)i + g.sy * j + g.sz * k + g.sv * v;
  Unew[c] = Uold[c];
}

inline unsigned cdiv(long long a, int b) { return (unsigned)((a + b - 1) / b); }

// k_mprim over all cells in storage order
template <int NDIM>
void launch_mprim(const Geo& g, const Geo& gq, const Phys& P, const double* U, float* Q,
                  float* rho, double* rho64, float* vel, double* pr, float* pp, float* mu,
                  float* nrg, float* Cc, float* T, float* lo, unsigned long long* red,
                  cudaStream_t st) {
  const dim3 qg(cdiv((long long)g.ngi * g.ngj, 256), 1, g.ngk), qb(256);
  k_mprim<NDIM><<<qg, qb, 0, st>>>(g, gq, P, U, Q, rho, rho64, vel, pr, pp, mu, nrg, Cc, T, lo,
                                   red);
}

Prim3Out prim3_out(const Phys& P, const MixedBufs& b, bool all_outputs) {
  const bool visc = all_outputs || P.visc, ceq = all_outputs || P.ceq;
  return Prim3Out{b.Q, b.rho32, b.vel32, b.p32, visc ? b.mu32 : nullptr, ceq ? b.nrg : nullptr,
                  ceq ? b.C : nullptr, ceq ? b.plo : nullptr, b.rho64};
}

// the 3D primitive pass over all cells (shell = false) or the ghost cells only
void launch_mprim3(const Geo& g, const Phys& P, const MixedBufs& b, const double* U,
                   bool all_outputs, unsigned long long* red, cudaStream_t st,
                   bool shell = false) {
  const Prim3Out O = prim3_out(P, b, all_outputs);
  if (shell) {
    const unsigned nb = cdiv(fst_shell_count(g), 256);
    switch (g.ns) {
      case 1: k_mprim3_shell<1><<<nb, 256, 0, st>>>(g, b.gq, P, U, O); break;
      case 2: k_mprim3_shell<2><<<nb, 256, 0, st>>>(g, b.gq, P, U, O); break;
      case 3: k_mprim3_shell<3><<<nb, 256, 0, st>>>(g, b.gq, P, U, O); break;
      case 4: k_mprim3_shell<4><<<nb, 256, 0, st>>>(g, b.gq, P, U, O); break;
      case 5: k_mprim3_shell<5><<<nb, 256, 0, st>>>(g, b.gq, P, U, O); break;
      default: k_mprim3_shell<0><<<nb, 256, 0, st>>>(g, b.gq, P, U, O); break;
    }
    return;
  }
  const dim3 qg(cdiv((long long)g.ngi * g.ngj, 256), 1, g.ngk), qb(256);
  switch (g.ns) {
    case 1: k_mprim3<1><<<qg, qb, 0, st>>>(g, b.gq, P, U, O, red); break;
    case 2: k_mprim3<2><<<qg, qb, 0, st>>>(g, b.gq, P, U, O, red); break;
    case 3: k_mprim3<3><<<qg, qb, 0, st>>>(g, b.gq, P, U, O, red); break;
    case 4: k_mprim3<4><<<qg, qb, 0, st>>>(g, b.gq, P, U, O, red); break;
    case 5: k_mprim3<5><<<qg, qb, 0, st>>>(g, b.gq, P, U, O, red); break;
    default: k_mprim3<0><<<qg, qb, 0, st>>>(g, b.gq, P, U, O, red); break;
  }
}

// Launch the fused 2D RHS for a compile-time variable count.
template <int NV, bool HYB>
void launch_rhs(const Geo& g, const Phys& P, const MixedView& M, const unsigned long long* red,
                const unsigned char* smap, const double* Uold, double* Unew, double coef,
                double* Rout, cudaStream_t st) {
  const dim3 blk(TX, TY, 1);
  const dim3 grd(cdiv(g.nci, TX - 1), cdiv(g.ncj, TY - 1), 1);
  k_mrhs2d<NV, HYB><<<grd, blk, 0, st>>>(g, P, M, red, smap, Uold, Unew, coef, Rout);
}

template <bool HYB>
void dispatch_rhs(const Geo& g, const Phys& P, const MixedView& M, const unsigned long long* red,
                  const unsigned char* smap, const double* Uold, double* Unew, double coef,
                  double* Rout, cudaStream_t st) {
  switch (g.nv) {
    case 4: launch_rhs<4, HYB>(g, P, M, red, smap, Uold, Unew, coef, Rout, st); break;
    case 5: launch_rhs<5, HYB>(g, P, M, red, smap, Uold, Unew, coef, Rout, st); break;
    case 6: launch_rhs<6, HYB>(g, P, M, red, smap, Uold, Unew, coef, Rout, st); break;
    case 7: launch_rhs<7, HYB>(g, P, M, red, smap, Uold, Unew, coef, Rout, st); break;
    case 8: launch_rhs<8, HYB>(g, P, M, red, smap, Uold, Unew, coef, Rout, st); break;
    case 9: launch_rhs<9, HYB>(g, P, M, red, smap, Uold, Unew, coef, Rout, st); break;
    default: launch_rhs<NVMAX, HYB>(g, P, M, red, smap, Uold, Unew, coef, Rout, st); break;
  }
}

}  // namespace

size_t fst_mixed_work_doubles_per_cell(const fst_config& cf, const Geo& g) {
  // floats: Q nv, rho, vel ndim, mu, nrg, C 5, T; doubles: p, rho and the
  // FP64 secondary outputs (rho, p, vel, T); hybrid: 3 map bytes
  const size_t fl = g.nv + 1 + g.ndim + 1 + 1 + 5 + 1 + 2;
  // generalized grids: 9 FP64 metrics + 18 FP32 metric pairs
  const size_t gen = cf.grid_type == FST_GRID_GENERALIZED ? 9 + 9 : 0;
  return (fl + 1) / 2 + 1 + (size_t)(g.ndim + 3) + 1 + gen;
}

int fst_mixed_alloc(const fst_config& cf, const Geo& g, MixedBufs& b, const fst_alloc_fn& alloc,
                    std::string* why) {
  b.gq = fst_prim_geo(g);
  const size_t n = (size_t)b.gq.sv;  // primitive arrays
  const size_t ns = (size_t)g.sv;    // FP64 secondary outputs (state layout)
  int rc = 0;
  auto A = [&](void** p, size_t bytes) {
    if (!rc) rc = alloc(p, bytes);
  };
  A((void**)&b.Q, sizeof(float) * n * g.nv);
  A((void**)&b.rho32, sizeof(float) * n);
  A((void**)&b.vel32, sizeof(float) * n * g.ndim);
  if (g.ndim == 3) A((void**)&b.p32, sizeof(float) * n * 2);
  else A((void**)&b.p64, sizeof(double) * n);
  if (cf.buoyancy) A((void**)&b.rho64, sizeof(double) * n);
  if (cf.visc && g.ndim == 3) A((void**)&b.mu32, sizeof(float) * n);
  if (cf.visc && g.ndim == 2) A((void**)&b.T32, sizeof(float) * n);
  if (cf.ceq) {
    A((void**)&b.nrg, sizeof(float) * n);
    A((void**)&b.C, sizeof(float) * n * 5);
    A((void**)&b.plo, sizeof(float) * n * 5);
  }
  A((void**)&b.rho, sizeof(double) * ns);
  A((void**)&b.pr, sizeof(double) * ns);
  A((void**)&b.vel, sizeof(double) * ns * g.ndim);
  A((void**)&b.T, sizeof(double) * ns);
  A((void**)&b.red, sizeof(unsigned long long) * 2);
  A((void**)&b.counters, sizeof(unsigned long long) * 8);
  A((void**)&b.dev_err, sizeof(unsigned int));
  if (cf.grid_type == FST_GRID_GENERALIZED) {
    A((void**)&b.met64, sizeof(double) * ns * 9);
    A((void**)&b.metf, sizeof(float) * n * 18);
  }
  // fused 3D stages: cartesian grids whose species fit one species launch
  // (FST_MIXED_UNFUSED=1 runs the separate primitive pass instead, which
  // gives the same bits; the tests compare the two)
  const char* unf = getenv("FST_MIXED_UNFUSED");
  b.fused = g.ndim == 3 && cf.grid_type == FST_GRID_CARTESIAN && g.ns <= 5 &&
            !(unf && unf[0] == '1');
  b.fused_for = nullptr;
  if (b.fused) {
    PrimSet& a = b.alt;
    A((void**)&a.Q, sizeof(float) * n * g.nv);
    A((void**)&a.rho32, sizeof(float) * n);
    A((void**)&a.vel32, sizeof(float) * n * 3);
    A((void**)&a.p32, sizeof(float) * n * 2);
    if (cf.buoyancy) A((void**)&a.rho64, sizeof(double) * n);
    if (cf.visc) A((void**)&a.mu32, sizeof(float) * n);
    if (cf.ceq) {
      A((void**)&a.nrg, sizeof(float) * n);
      A((void**)&a.C, sizeof(float) * n * 5);
      A((void**)&a.plo, sizeof(float) * n * 5);
    }
    A((void**)&a.red, sizeof(unsigned long long) * 2);
  }
  if (!rc && cf.mode == FST_MODE_HYBRID) rc = fst_hybrid_alloc(cf, g, b, alloc);
  if (!rc) rc = fst_mixed3d_prepare(g, b, why);
  return rc;
}

void fst_mixed_swap(MixedBufs& b) {
  PrimSet& a = b.alt;
  std::swap(b.Q, a.Q);
  std::swap(b.rho32, a.rho32);
  std::swap(b.vel32, a.vel32);
  std::swap(b.mu32, a.mu32);
  std::swap(b.nrg, a.nrg);
  std::swap(b.C, a.C);
  std::swap(b.p32, a.p32);
  std::swap(b.plo, a.plo);
  std::swap(b.rho64, a.rho64);
  std::swap(b.maps3d, a.maps3d);
  std::swap(b.red, a.red);
}

cudaError_t fst_mixed_canary(const Geo& g, const MixedBufs& b, cudaStream_t st) {
  const size_t n = (size_t)b.gq.sv;
  const PrimSet& a = b.alt;
  const struct {
    void* p;
    size_t bytes;
  } f[] = {{b.Q, sizeof(float) * n * g.nv}, {b.rho32, sizeof(float) * n},
           {b.vel32, sizeof(float) * n * g.ndim}, {b.mu32, sizeof(float) * n},
           {b.T32, sizeof(float) * n}, {b.nrg, sizeof(float) * n},
           {b.C, sizeof(float) * n * 5}, {b.p32, sizeof(float) * n * 2},
           {b.p64, sizeof(double) * n}, {b.metf, sizeof(float) * n * 18},
           {b.plo, sizeof(float) * n * 5}, {a.Q, sizeof(float) * n * g.nv},
           {a.rho32, sizeof(float) * n}, {a.vel32, sizeof(float) * n * 3},
           {a.mu32, sizeof(float) * n}, {a.nrg, sizeof(float) * n},
           {a.C, sizeof(float) * n * 5}, {a.p32, sizeof(float) * n * 2},
           {a.plo, sizeof(float) * n * 5}};
  cudaError_t e = cudaSuccess;
  for (const auto& x : f)
    if (x.p && e == cudaSuccess) e = cudaMemsetAsync(x.p, 0xFF, x.bytes, st);
  return e;
}

int fst_mixed_stage(const Geo& g, const Phys& P, const fst_config& cf, MixedBufs& b,
                    const double* Uin, const double* Uold, double* Unew, double coef, double* Rout,
                    bool ghosts, cudaStream_t st, Prof* prof) {
  int n = 0;
  // Fused 3D stages: the previous stage left the primitives of Uin's interior
  // (and the C-equation maxima) in the current set; only the ghost cells,
  // just filled by the boundary conditions, remain.  Otherwise (first stage
  // after the state was set, a bare RHS) the whole primitive pass runs.
  const bool fuse = b.fused && !Rout && !b.metf;
  const bool have = fuse && b.fused_for == Uin;
  if (!fuse) b.fused_for = nullptr;
  if (P.ceq && !have) {
    fst_fill_keys(b.red, 2, FST_KEY_LOWEST, st);
    ++n;
  }
  if (fuse) {
    fst_fill_keys(b.alt.red, 2, FST_KEY_LOWEST, st);
    ++n;
  }
  const MixedView M{b.Q, b.rho32, b.vel32, b.p64,  b.mu32,
                    b.nrg, b.C, b.T32, b.rho64, b.p32, b.plo};
  if (g.ndim == 3 && have) {
    FST_LAUNCH(prof, "mprim3d_shell", st, n, launch_mprim3(g, P, b, Uin, false, nullptr, st, true));
  } else if (g.ndim == 3) {
    FST_LAUNCH(prof, "mprim3d", st, n,
               launch_mprim3(g, P, b, Uin, false, P.ceq ? b.red : nullptr, st));
    if (b.metf)  // generalized grid: contravariant velocity for the face kernels
      FST_LAUNCH(prof, "gen_tvel", st, n, fst_mixedgen_tvel(g, b.gq, b.metf, b.vel32, st));
  } else {
    FST_LAUNCH(prof, "mprim2d", st, n,
               launch_mprim<2>(g, b.gq, P, Uin, b.Q, b.rho32, b.rho64, b.vel32, b.p64, nullptr,
                               nullptr, P.ceq ? b.nrg : nullptr, P.ceq ? b.C : nullptr,
                               P.visc ? b.T32 : nullptr, P.ceq ? b.plo : nullptr,
                               P.ceq ? b.red : nullptr, st));
  }
  bool hyb = cf.mode == FST_MODE_HYBRID && b.hyb_active;
  const unsigned char* smooth = b.smooth;
  if (hyb) {
    // classify once per time step (stage 1, or a bare RHS evaluation) and
    // reuse the map at stage 2; audit steps run full WENO5 and only compare
    // the classifier's decisions with the smoothness labels
    const bool audit = b.audit_every > 0 && b.stage != 0 && (b.step % b.audit_every) == 0;
    const bool due = b.stage == 0 || audit || !b.classified ||
                     (b.stage == 1 && b.step % b.classify_every == 0);
    if (due) {
      n += fst_hybrid_classify(b.gq, P, b, M, st, prof, &smooth, audit);
      b.classified = true;
    }
    if (audit) hyb = false;
  }
  if (g.ndim == 3)
    n += fst_mixed3d_rhs(g, P, b, M, smooth, Uold, Unew, coef, Rout, st, prof, hyb, fuse);
  else if (hyb)
    FST_LAUNCH(prof, "mrhs2d_hybrid", st, n,
               dispatch_rhs<true>(g, P, M, b.red, smooth, Uold, Unew, coef, Rout, st));
  else
    FST_LAUNCH(prof, "mrhs2d", st, n,
               dispatch_rhs<false>(g, P, M, b.red, nullptr, Uold, Unew, coef, Rout, st));
  if (ghosts && !Rout)
    FST_LAUNCH(prof, "mghost", st, n,
               k_mghost<<<cdiv(fst_shell_count(g) * g.nvt, 256), 256, 0, st>>>(
                   g, fst_shell_count(g), Uold, Unew));
  if (fuse) {  // the next stage reads what this one wrote into the other set
    fst_mixed_swap(b);
    b.fused_for = Unew;
  }
  return n;
}

int fst_mixed_upload(const Geo& g, const Phys& P, MixedBufs& b, const double* Uh, double* U,
                     cudaStream_t st, Prof* prof) {
  if (g.ndim != 3 || !b.fused || b.metf || g.ns < 1 || g.ns > 5) return -1;
  int n = 0;
  if (P.ceq) fst_fill_keys(b.red, 2, FST_KEY_LOWEST, st);
  const Prim3Out O = prim3_out(P, b, false);
  unsigned long long* red = P.ceq ? b.red : nullptr;
  const dim3 qg(cdiv((long long)g.ngi * g.ngj, 256), 1, g.ngk), qb(256);
  auto launch = [&]() {
    switch (g.ns) {
      case 1: k_mupload3<1><<<qg, qb, 0, st>>>(g, b.gq, P, Uh, U, O, red); break;
      case 2: k_mupload3<2><<<qg, qb, 0, st>>>(g, b.gq, P, Uh, U, O, red); break;
      case 3: k_mupload3<3><<<qg, qb, 0, st>>>(g, b.gq, P, Uh, U, O, red); break;
      case 4: k_mupload3<4><<<qg, qb, 0, st>>>(g, b.gq, P, Uh, U, O, red); break;
      default: k_mupload3<5><<<qg, qb, 0, st>>>(g, b.gq, P, Uh, U, O, red); break;
    }
  };
  FST_LAUNCH(prof, "mupload3d", st, n, launch());
  b.fused_for = U;
  return n + (P.ceq ? 1 : 0);  // and the key fill
}

int fst_mixed_secondary(const Geo& g, const Phys& P, const MixedBufs& b, const double* U,
                        cudaStream_t st, const double** rho, const double** pr, const double** vel,
                        const double** T) {
  int n;
  if (g.ndim == 3) {
    Plain3DBufs p3{};
    p3.rho = b.rho; p3.pr = b.pr; p3.vel = b.vel; p3.T = b.T;
    n = fst_plain3d_secondary(g, P, p3, U, st);
  } else {
    Plain2DBufs p2{};
    p2.rho = b.rho; p2.pr = b.pr; p2.vel = b.vel; p2.T = b.T;
    n = fst_plain2d_secondary(g, P, p2, U, st);
  }
  *rho = b.rho;
  *pr = b.pr;
  *vel = b.vel;
  *T = b.T;
  return n;
}

int fst_mixed_prims(const Geo& g, const Phys& P, const fst_config& cf, const MixedBufs& b,
                    const double* U, cudaStream_t st) {
  (void)cf;
  if (g.ndim == 3)
    launch_mprim3(g, P, b, U, true, nullptr, st);
  else
    launch_mprim<2>(g, b.gq, P, U, b.Q, b.rho32, b.rho64, b.vel32, b.p64, nullptr, nullptr, b.nrg,
                    b.C, b.T32, b.plo, nullptr, st);
  return 1;
}

double fst_mixed_flagged_fraction(const MixedBufs& b, cudaStream_t st) {
  if (!b.hyb_active || !b.counters) return 0.0;
  unsigned long long h[2] = {0, 0};
  if (cudaMemcpyAsync(h, b.counters, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return 0.0;
  return h[0] ? (double)h[1] / (double)h[0] : 0.0;
}
