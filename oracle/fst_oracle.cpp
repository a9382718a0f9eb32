// fst_oracle.cpp — CPU oracle for the FIESTA RHS + RK path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU path is compared
// against; it is loaded by tests/, by __graft_entry__.smoke() and by the CPU
// baseline leg of bench.py, and by nothing else.  It is never linked into the
// product library.
//
// It restates, in plain serial/OpenMP C++, the reference's FP64 kernel
// sequence operation for operation:
//   - cart3d_func::compute      (src/cart3d.cpp:220-298)
//   - cart2d_func::compute      (src/cart2d.cpp:151-237), preStep (:147-149),
//                               with the WENO5 / centred / QUICK 2D fluxes
//   - gen3d_func::compute / gen2d_func::compute (src/gen3d.cpp:338-370,
//     src/gen2d.cpp:103-130) and their preSim metrics (src/metric.hpp)
//   - rkAdvance                 (src/rk.cpp:28-70)
//   - applyBCs / bc_gen / bc_*Per (src/bc.cpp:33-249)
// Each kernel function below names the reference functor it follows.  The
// expression order inside each one is the reference's, because FP64 results
// are compared bit for bit; build with -ffp-contract=off (aarch64 GCC
// contracts a*b+c into FMA by default).
//
// Storage is LayoutRight (v fastest, then k, j, i), the layout Kokkos gives
// the reference's host (Serial/OpenMP) build (src/kokkosTypes.hpp:40); the
// ABI (fst.h) exchanges LayoutLeft arrays and they are repacked at the edge.
//
// Parity pin: tests/test_oracle_golden.py checks this oracle against golden
// vectors produced by the reference's own kernel sources compiled here
// (oracle/ref_build.sh), and against the reference's BC known-answer tests
// (tests/bc_outflow.cpp, bc_reflective.cpp, bc_hydrostatic.cpp, test.cpp).

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/fst.h"

namespace {

struct Oracle {
  fst_config cf;
  int ng, nci, ncj, nck, ngi, ngj, ngk, ns, nv, nvt, ndim;
  double dx, dy, dz, dt;
  std::vector<double> cd;  // device config array: src/cart3d.cpp:152-171
  double dxmag;            // src/cart3d.cpp:173 (3D only)

  std::vector<double> var, tmp1, dvar;
  std::vector<double> p, T, rho, vel;
  std::vector<double> fluxx, fluxy, fluxz;
  std::vector<double> stress;            // 3D: (i,j,k,6)
  std::vector<double> stressx, stressy;  // 2D: (i,j,2,2)
  std::vector<double> qx, qy;            // 2D heat flux
  std::vector<double> gradRho;           // 3D: 5 comps, 2D: 4 comps
  std::vector<double> mFlux;             // 3D: (3,3,i,j,k,3), 2D m: (2,2,i,j,2)
  // generalized grids (src/gen3d.cpp, src/gen2d.cpp)
  bool gen = false;
  int scheme = 1;                        // 2D advection scheme (cf.scheme)
  double fdz = 1;                        // dz passed to calculateFluxesG
  std::vector<double> met;               // (i,j,k,a,b), a,b < ndim
  std::vector<double> nodes;             // (ni,nj,nk,3), LayoutLeft as given
  int ni = 0, nj = 0, nk = 0;
  double last_maxS = 0, last_maxCh = 0;
  std::string err;

  // ---- LayoutRight index helpers -------------------------------------
  inline size_t c3(int i, int j, int k) const {
    return ((size_t)i * ngj + j) * ngk + k;
  }
  inline double& V(int i, int j, int k, int v) { return var[c3(i, j, k) * nvt + v]; }
  inline double& D(int i, int j, int k, int v) { return dvar[c3(i, j, k) * nvt + v]; }
  inline double& P(int i, int j, int k) { return p[c3(i, j, k)]; }
  inline double& RHO(int i, int j, int k) { return rho[c3(i, j, k)]; }
  inline double& TT(int i, int j, int k) { return T[c3(i, j, k)]; }
  inline double& VEL(int i, int j, int k, int d) { return vel[c3(i, j, k) * ndim + d]; }
  inline double& STR(int i, int j, int k, int c) { return stress[c3(i, j, k) * 6 + c]; }
  inline double& GR(int i, int j, int k, int n) {
    return gradRho[c3(i, j, k) * (ndim == 3 ? 5 : 4) + n];
  }
  inline double& MF3(int f, int d, int i, int j, int k, int w) {
    return mFlux[((size_t)(f * 3 + d) * ngi * ngj * ngk + c3(i, j, k)) * 3 + w];
  }
  // 2D arrays (k == 0)
  inline double& SX(int i, int j, int a, int b) { return stressx[(c3(i, j, 0) * 2 + a) * 2 + b]; }
  inline double& SY(int i, int j, int a, int b) { return stressy[(c3(i, j, 0) * 2 + a) * 2 + b]; }
  inline double& QX(int i, int j) { return qx[c3(i, j, 0)]; }
  inline double& QY(int i, int j) { return qy[c3(i, j, 0)]; }
  inline double& M2(int f, int d, int i, int j, int w) {
    return mFlux[((size_t)(f * 2 + d) * ngi * ngj + c3(i, j, 0)) * 2 + w];
  }

  // Loops over a box [b0,e0)x[b1,e1)x[b2,e2), the MDRange policies of the
  // reference.  Cells are independent inside each reference kernel, so the
  // OpenMP split does not change results.
  template <class F>
  void box(int b0, int e0, int b1, int e1, int b2, int e2, F&& f) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = b0; i < e0; ++i)
      for (int j = b1; j < e1; ++j)
        for (int k = b2; k < e2; ++k) f(i, j, k);
  }
  template <class F>
  double box_max(int b0, int e0, int b1, int e1, int b2, int e2, F&& f) {
    // Kokkos::Max starts from reduction_identity<double>::max() = -DBL_MAX;
    // `if (s > lmax) lmax = s` skips NaN.
    double gmax = -DBL_MAX;
#pragma omp parallel
    {
      double lmax = -DBL_MAX;
#pragma omp for collapse(2) schedule(static) nowait
      for (int i = b0; i < e0; ++i)
        for (int j = b1; j < e1; ++j)
          for (int k = b2; k < e2; ++k) {
            double s = f(i, j, k);
            if (s > lmax) lmax = s;
          }
#pragma omp critical
      {
        if (lmax > gmax) gmax = lmax;
      }
    }
    return gmax;
  }

  int init(const fst_config* c) {
    cf = *c;
    ndim = cf.ndim;
    ng = cf.ng;
    nci = cf.nci;
    ncj = cf.ncj;
    nck = ndim == 3 ? cf.nck : 1;
    ngi = nci + 2 * ng;
    ngj = ncj + 2 * ng;
    ngk = ndim == 3 ? nck + 2 * ng : 1;
    ns = cf.ns;
    nv = ndim == 3 ? 4 + ns : 3 + ns;  // src/input.cpp:401-408
    nvt = nv + (cf.ceq ? 5 : 0);        // src/input.cpp:411-414
    dx = cf.dx;
    dy = cf.dy;
    dz = ndim == 3 ? cf.dz : cf.dx;     // 2D: dz = dx (src/input.cpp:402)
    dt = cf.dt;
    cd.assign(6 + 3 * ns, 0.0);
    cd[0] = ns; cd[1] = dx; cd[2] = dy; cd[3] = dz; cd[4] = nv; cd[5] = ng;
    for (int s = 0; s < ns; ++s) {
      cd[6 + 3 * s] = cf.gamma[s];
      cd[7 + 3 * s] = cf.R / cf.M[s];
      cd[8 + 3 * s] = cf.mu[s];
    }
    dxmag = dx * dx + dy * dy + dz * dz;
    gen = cf.grid_type == FST_GRID_GENERALIZED;
    scheme = ndim == 2 && cf.scheme > 0 ? cf.scheme : 1;
    fdz = gen ? dx : dz;  // gen3d passes cf.dx as dz (src/gen3d.cpp:359)
    if (gen) {             // the modules compute advection and pressure only
      cf.visc = 0;
      cf.ceq = 0;
      cf.buoyancy = 0;
    }
    ni = nci + 1;
    nj = ncj + 1;
    nk = ndim == 3 ? nck + 1 : 1;
    size_t nc = (size_t)ngi * ngj * ngk;
    var.assign(nc * nvt, 0.0);
    tmp1.assign(nc * nvt, 0.0);
    dvar.assign(nc * nvt, 0.0);
    p.assign(nc, 0.0); T.assign(nc, 0.0); rho.assign(nc, 0.0);
    vel.assign(nc * ndim, 0.0);
    fluxx.assign(nc, 0.0); fluxy.assign(nc, 0.0);
    if (ndim == 3) fluxz.assign(nc, 0.0);
    if (gen) met.assign(nc * ndim * ndim, 0.0);
    if (cf.visc) {
      if (ndim == 3) stress.assign(nc * 6, 0.0);
      else { stressx.assign(nc * 4, 0.0); stressy.assign(nc * 4, 0.0);
             qx.assign(nc, 0.0); qy.assign(nc, 0.0); }
    }
    if (cf.ceq) {
      gradRho.assign(nc * (ndim == 3 ? 5 : 4), 0.0);
      mFlux.assign(ndim == 3 ? 27 * nc : 8 * nc, 0.0);
    }
    return FST_OK;
  }

  // ==================================================================
  // Boundary conditions — src/bc.cpp
  // ==================================================================
  // bc_gen::operator() (src/bc.cpp:42-130) on the face line through (i,j,k).
  void bc_gen(int type, int ih, int jh, int kh, int i, int j, int k) {
    auto U = [&](int a, int b, int c, int v) -> double& { return V(a, b, c, v); };
    if (type == FST_BC_OUTFLOW) {
      for (int v = 0; v < nvt; ++v)
        for (int n = 0; n < ng; ++n)
          U(i + ih * (n + 1), j + jh * (n + 1), k + kh * (n + 1), v) =
              U(i - ih * n, j - jh * n, k - kh * n, v);
    }
    if (type == FST_BC_REFLECTIVE || type == FST_BC_HYDROSTATIC) {
      for (int v = 0; v < nvt; ++v) {
        double reflect = 1.0;
        if (ih != 0 && v == 0) reflect = -1.0;
        if (jh != 0 && v == 1) reflect = -1.0;
        if (kh != 0 && v == 2) reflect = -1.0;
        for (int n = 0; n < ng; ++n)
          U(i + ih * (n + 1), j + jh * (n + 1), k + kh * (n + 1), v) =
              reflect * U(i - ih * n, j - jh * n, k - kh * n, v);
      }
    }
    if (type == FST_BC_NOSLIP) {
      for (int v = 0; v < nvt; ++v) {
        double reflect = 1.0;
        bool mom = (v == 0 || v == 1 || v == 2);
        if (ih != 0 && mom) reflect = -1.0;
        if (jh != 0 && mom) reflect = -1.0;
        if (kh != 0 && mom) reflect = -1.0;
        for (int n = 0; n < ng; ++n)
          U(i + ih * (n + 1), j + jh * (n + 1), k + kh * (n + 1), v) =
              reflect * U(i - ih * n, j - jh * n, k - kh * n, v);
      }
    }
    if (type == FST_BC_HYDROSTATIC) {
      // energy: linear extrapolation of internal energy (src/bc.cpp:92-123)
      const int edx = ndim, rdx = ndim + 1;
      for (int n = 0; n < ng; ++n) {
        int ig = i + ih * (n + 1), jg = j + jh * (n + 1), kg = k + kh * (n + 1);
        int i1 = ig - ih, j1 = jg - jh, k1 = kg - kh;
        int i2 = ig - 2 * ih, j2 = jg - 2 * jh, k2 = kg - 2 * kh;
        double ke = 0, ke1 = 0, ke2 = 0;
        for (int d = 0; d < ndim; ++d) {
          ke += 0.5 * (U(ig, jg, kg, d) * U(ig, jg, kg, d));
          ke1 += 0.5 * (U(i1, j1, k1, d) * U(i1, j1, k1, d));
          ke2 += 0.5 * (U(i2, j2, k2, d) * U(i2, j2, k2, d));
        }
        ke = ke / U(ig, jg, kg, rdx);
        ke1 = ke1 / U(i1, j1, k1, rdx);
        ke2 = ke2 / U(i2, j2, k2, rdx);
        U(ig, jg, kg, edx) =
            2 * (U(i1, j1, k1, edx) - ke1) - (U(i2, j2, k2, edx) - ke2) + ke;
      }
    }
  }

  // applyBCs (src/bc.cpp:179-249), non-MPI ordering: periodic x, y, z
  // self-copies (bc_xPer/yPer/zPer, :133-176), then face fills.
  void apply_bcs() {
    if (cf.xper) {
#pragma omp parallel for collapse(2)
      for (int j = 0; j < ngj; ++j)
        for (int k = 0; k < ngk; ++k)
          for (int v = 0; v < nvt; ++v)
            for (int g = 0; g < ng; ++g) {
              V(g, j, k, v) = V(nci + g, j, k, v);
              V(nci + ng + g, j, k, v) = V(ng + g, j, k, v);
            }
    }
    if (cf.yper) {
#pragma omp parallel for collapse(2)
      for (int i = 0; i < ngi; ++i)
        for (int k = 0; k < ngk; ++k)
          for (int v = 0; v < nvt; ++v)
            for (int g = 0; g < ng; ++g) {
              V(i, g, k, v) = V(i, ncj + g, k, v);
              V(i, ncj + ng + g, k, v) = V(i, ng + g, k, v);
            }
    }
    if (ndim == 3 && cf.zper) {
#pragma omp parallel for collapse(2)
      for (int i = 0; i < ngi; ++i)
        for (int j = 0; j < ngj; ++j)
          for (int v = 0; v < nvt; ++v)
            for (int g = 0; g < ng; ++g) {
              V(i, j, g, v) = V(i, j, nck + g, v);
              V(i, j, nck + ng + g, v) = V(i, j, ng + g, v);
            }
    }
    if (!cf.xper) {
      box(ng, ng + 1, 0, ngj, 0, ngk, [&](int i, int j, int k) { bc_gen(cf.bc_xmin, -1, 0, 0, i, j, k); });
      box(ng + nci - 1, ng + nci, 0, ngj, 0, ngk, [&](int i, int j, int k) { bc_gen(cf.bc_xmax, 1, 0, 0, i, j, k); });
    }
    if (!cf.yper) {
      box(0, ngi, ng, ng + 1, 0, ngk, [&](int i, int j, int k) { bc_gen(cf.bc_ymin, 0, -1, 0, i, j, k); });
      box(0, ngi, ng + ncj - 1, ng + ncj, 0, ngk, [&](int i, int j, int k) { bc_gen(cf.bc_ymax, 0, 1, 0, i, j, k); });
    }
    if (ndim == 3 && !cf.zper) {
      box(0, ngi, 0, ngj, ng, ng + 1, [&](int i, int j, int k) { bc_gen(cf.bc_zmin, 0, 0, -1, i, j, k); });
      box(0, ngi, 0, ngj, ng + nck - 1, ng + nck, [&](int i, int j, int k) { bc_gen(cf.bc_zmax, 0, 0, 1, i, j, k); });
    }
  }

  // ==================================================================
  // 3D kernels
  // ==================================================================
  // calculateRhoPT3D (src/secondary.hpp:109-151)
  void rhoPT3D(int i, int j, int k) {
    double gamma, gammas, Rs, Cp = 0, Cv = 0;
    RHO(i, j, k) = 0.0;
    for (int s = 0; s < ns; ++s) RHO(i, j, k) = RHO(i, j, k) + V(i, j, k, 4 + s);
    for (int s = 0; s < ns; ++s) {
      gammas = cd[6 + 3 * s];
      Rs = cd[6 + 3 * s + 1];
      Cp = Cp + (V(i, j, k, 4 + s) / RHO(i, j, k)) * (gammas * Rs / (gammas - 1));
      Cv = Cv + (V(i, j, k, 4 + s) / RHO(i, j, k)) * (Rs / (gammas - 1));
    }
    gamma = Cp / Cv;
    P(i, j, k) = (gamma - 1) * (V(i, j, k, 3) - (0.5 / RHO(i, j, k)) *
                                                    (V(i, j, k, 0) * V(i, j, k, 0) +
                                                     V(i, j, k, 1) * V(i, j, k, 1) +
                                                     V(i, j, k, 2) * V(i, j, k, 2)));
    TT(i, j, k) = P(i, j, k) / ((Cp - Cv) * RHO(i, j, k));
  }
  // computeVelocity3D (src/velocity.hpp:68-83)
  void velocity3D(int i, int j, int k) {
    VEL(i, j, k, 0) = V(i, j, k, 0) / RHO(i, j, k);
    VEL(i, j, k, 1) = V(i, j, k, 1) / RHO(i, j, k);
    VEL(i, j, k, 2) = V(i, j, k, 2) / RHO(i, j, k);
  }

  // calculateFluxesG::weno (src/flux.hpp:241-266): float-literal constants.
  static inline double weno3(double f1, double f2, double f3, double f4, double f5) {
    const double eps = 0.000001;
    double b1, b2, b3, w1, w2, w3, p1, p2, p3, a1, a2;
    a1 = f1 - 2.0f * f2 + f3;
    a2 = f1 - 4.0f * f2 + 3.0f * f3;
    b1 = (13.0f / 12.0f) * a1 * a1 + (0.25f) * a2 * a2;
    a1 = f2 - 2.0 * f3 + f4;
    a2 = f2 - f4;
    b2 = (13.0f / 12.0f) * a1 * a1 + (0.25f) * a2 * a2;
    a1 = f3 - 2.0 * f4 + f5;
    a2 = 3.0 * f3 - 4.0 * f4 + f5;
    b3 = (13.0f / 12.0f) * a1 * a1 + (0.25f) * a2 * a2;
    a1 = eps + b1;
    w1 = (0.1f) / (a1 * a1);
    a1 = eps + b2;
    w2 = (0.6f) / (a1 * a1);
    a1 = eps + b3;
    w3 = (0.3f) / (a1 * a1);
    p1 = (1.0f / 3.0f) * f1 + (-7.0f / 6.0f) * f2 + (11.0f / 6.0f) * f3;
    p2 = (-1.0f / 6.0f) * f2 + (5.0f / 6.0f) * f3 + (1.0f / 3.0f) * f4;
    p3 = (1.0f / 3.0f) * f3 + (5.0f / 6.0f) * f4 + (-1.0f / 6.0f) * f5;
    return (w1 * p1 + w2 * p2 + w3 * p3) / (w1 + w2 + w3);
  }

  // calculateFluxesG::operator() (src/flux.hpp:268-309)
  void fluxes3D(int i, int j, int k, int v) {
    double ur, vr, wr, f1, f2, f3, f4, f5, f6;
    auto q = [&](int a, int b, int c) { return V(a, b, c, v) + (v == 3) * P(a, b, c); };
    f1 = q(i + 3, j, k); f2 = q(i + 2, j, k); f3 = q(i + 1, j, k);
    f4 = q(i, j, k); f5 = q(i - 1, j, k); f6 = q(i - 2, j, k);
    ur = (-VEL(i + 2, j, k, 0) + 7.0f * VEL(i + 1, j, k, 0) + 7.0f * VEL(i, j, k, 0) -
          VEL(i - 1, j, k, 0)) / 12.0f;
    if (ur < 0.0) fluxx[c3(i, j, k)] = ur * weno3(f1, f2, f3, f4, f5) / dx;
    else          fluxx[c3(i, j, k)] = ur * weno3(f6, f5, f4, f3, f2) / dx;

    f1 = q(i, j + 3, k); f2 = q(i, j + 2, k); f3 = q(i, j + 1, k);
    f4 = q(i, j, k); f5 = q(i, j - 1, k); f6 = q(i, j - 2, k);
    vr = (-VEL(i, j + 2, k, 1) + 7.0f * VEL(i, j + 1, k, 1) + 7.0f * VEL(i, j, k, 1) -
          VEL(i, j - 1, k, 1)) / 12.0f;
    if (vr < 0.0) fluxy[c3(i, j, k)] = vr * weno3(f1, f2, f3, f4, f5) / dy;
    else          fluxy[c3(i, j, k)] = vr * weno3(f6, f5, f4, f3, f2) / dy;

    f1 = q(i, j, k + 3); f2 = q(i, j, k + 2); f3 = q(i, j, k + 1);
    f4 = q(i, j, k); f5 = q(i, j, k - 1); f6 = q(i, j, k - 2);
    wr = (-VEL(i, j, k + 2, 2) + 7.0f * VEL(i, j, k + 1, 2) + 7.0f * VEL(i, j, k, 2) -
          VEL(i, j, k - 1, 2)) / 12.0f;
    if (wr < 0.0) fluxz[c3(i, j, k)] = wr * weno3(f1, f2, f3, f4, f5) / fdz;
    else          fluxz[c3(i, j, k)] = wr * weno3(f6, f5, f4, f3, f2) / fdz;
  }
  // advect3D (src/advect.hpp:39-61)
  void advect3D(int i, int j, int k, int v) {
    double res = -((fluxx[c3(i, j, k)] - fluxx[c3(i - 1, j, k)]) +
                   (fluxy[c3(i, j, k)] - fluxy[c3(i, j - 1, k)]) +
                   (fluxz[c3(i, j, k)] - fluxz[c3(i, j, k - 1)]));
    D(i, j, k, v) = res;
  }
  // applyPressureGradient3D (src/presgrad.hpp:44-71); note dz = cd(2)
  void presgrad3D(int i, int j, int k) {
    double dx_ = cd[1], dy_ = cd[2], dz_ = cd[2];
    double dxp = (P(i - 2, j, k) - 8.0 * P(i - 1, j, k) + 8.0 * P(i + 1, j, k) - P(i + 2, j, k)) / (12.0 * dx_);
    double dyp = (P(i, j - 2, k) - 8.0 * P(i, j - 1, k) + 8.0 * P(i, j + 1, k) - P(i, j + 2, k)) / (12.0 * dy_);
    double dzp = (P(i, j, k - 2) - 8.0 * P(i, j, k - 1) + 8.0 * P(i, j, k + 1) - P(i, j, k + 2)) / (12.0 * dz_);
    D(i, j, k, 0) = D(i, j, k, 0) - dxp;
    D(i, j, k, 1) = D(i, j, k, 1) - dyp;
    D(i, j, k, 2) = D(i, j, k, 2) - dzp;
  }
  // computeBuoyancy3D (src/buoyancy.hpp:22-47)
  void buoyancy3D(int i, int j, int k) {
    double vv = V(i, j, k, 1) / RHO(i, j, k);
    double rhop = RHO(i, j, k) - cf.rho_ref;
    double f = -cf.g_accel * rhop;
    D(i, j, k, 1) += f;
    D(i, j, k, 3) += vv * f;
  }
  // calculateStressTensor{x,y,z}3dv (src/viscosity.hpp:416-459, 499-541, 581-624)
  void stress3D(int dir, int i, int j, int k) {
    const int ih = dir == 0, jh = dir == 1, kh = dir == 2;
    double dx_ = cd[1], dy_ = cd[2], dz_ = cd[3];
    double dudx, dudy, dudz, dvdx, dvdy, dvdz, dwdx, dwdy, dwdz, mu = 0.0;
    for (int s = 0; s < ns; ++s)
      mu += ((V(i + ih, j + jh, k + kh, 4 + s) / RHO(i + ih, j + jh, k + kh) +
              V(i, j, k, 4 + s) / RHO(i, j, k)) / 2.0) * cd[6 + 3 * s + 2];
    auto U = [&](int a, int b, int c, int d) { return VEL(a, b, c, d); };
    if (dir == 0) {
      dudx = (U(i + 1, j, k, 0) - U(i, j, k, 0)) / dx_;
      dvdx = (U(i + 1, j, k, 1) - U(i, j, k, 1)) / dx_;
      dwdx = (U(i + 1, j, k, 2) - U(i, j, k, 2)) / dx_;
      dudy = ((U(i + 1, j + 1, k, 0) + U(i, j + 1, k, 0)) - (U(i + 1, j - 1, k, 0) + U(i, j - 1, k, 0))) / (4 * dy_);
      dvdy = ((U(i + 1, j + 1, k, 1) + U(i, j + 1, k, 1)) - (U(i + 1, j - 1, k, 1) + U(i, j - 1, k, 1))) / (4 * dy_);
      dwdy = ((U(i + 1, j + 1, k, 2) + U(i, j + 1, k, 2)) - (U(i + 1, j - 1, k, 2) + U(i, j - 1, k, 2))) / (4 * dy_);
      dudz = ((U(i + 1, j, k + 1, 0) + U(i, j, k + 1, 0)) - (U(i + 1, j, k - 1, 0) + U(i, j, k - 1, 0))) / (4 * dz_);
      dvdz = ((U(i + 1, j, k + 1, 1) + U(i, j, k + 1, 1)) - (U(i + 1, j, k - 1, 1) + U(i, j, k - 1, 1))) / (4 * dz_);
      dwdz = ((U(i + 1, j, k + 1, 2) + U(i, j, k + 1, 2)) - (U(i + 1, j, k - 1, 2) + U(i, j, k - 1, 2))) / (4 * dz_);
    } else if (dir == 1) {
      dudx = ((U(i + 1, j + 1, k, 0) + U(i + 1, j, k, 0)) - (U(i - 1, j + 1, k, 0) + U(i - 1, j, k, 0))) / (4 * dx_);
      dvdx = ((U(i + 1, j + 1, k, 1) + U(i + 1, j, k, 1)) - (U(i - 1, j + 1, k, 1) + U(i - 1, j, k, 1))) / (4 * dx_);
      dwdx = ((U(i + 1, j + 1, k, 2) + U(i + 1, j, k, 2)) - (U(i - 1, j + 1, k, 2) + U(i - 1, j, k, 2))) / (4 * dx_);
      dudy = (U(i, j + 1, k, 0) - U(i, j, k, 0)) / dy_;
      dvdy = (U(i, j + 1, k, 1) - U(i, j, k, 1)) / dy_;
      dwdy = (U(i, j + 1, k, 2) - U(i, j, k, 2)) / dy_;
      dudz = ((U(i, j + 1, k + 1, 0) + U(i, j, k + 1, 0)) - (U(i, j + 1, k - 1, 0) + U(i, j, k - 1, 0))) / (4 * dz_);
      dvdz = ((U(i, j + 1, k + 1, 1) + U(i, j, k + 1, 1)) - (U(i, j + 1, k - 1, 1) + U(i, j, k - 1, 1))) / (4 * dz_);
      dwdz = ((U(i, j + 1, k + 1, 2) + U(i, j, k + 1, 2)) - (U(i, j + 1, k - 1, 2) + U(i, j, k - 1, 2))) / (4 * dz_);
    } else {
      dudx = ((U(i + 1, j, k + 1, 0) + U(i + 1, j, k, 0)) - (U(i - 1, j, k + 1, 0) + U(i - 1, j, k, 0))) / (4 * dx_);
      dvdx = ((U(i + 1, j, k + 1, 1) + U(i + 1, j, k, 1)) - (U(i - 1, j, k + 1, 1) + U(i - 1, j, k, 1))) / (4 * dx_);
      dwdx = ((U(i + 1, j, k + 1, 2) + U(i + 1, j, k, 2)) - (U(i - 1, j, k + 1, 2) + U(i - 1, j, k, 2))) / (4 * dx_);
      dudy = ((U(i, j + 1, k + 1, 0) + U(i, j + 1, k, 0)) - (U(i, j - 1, k + 1, 0) + U(i, j - 1, k, 0))) / (4 * dy_);
      dvdy = ((U(i, j + 1, k + 1, 1) + U(i, j + 1, k, 1)) - (U(i, j - 1, k + 1, 1) + U(i, j - 1, k, 1))) / (4 * dy_);
      dwdy = ((U(i, j + 1, k + 1, 2) + U(i, j + 1, k, 2)) - (U(i, j - 1, k + 1, 2) + U(i, j - 1, k, 2))) / (4 * dy_);
      dudz = (U(i, j, k + 1, 0) - U(i, j, k, 0)) / dz_;
      dvdz = (U(i, j, k + 1, 1) - U(i, j, k, 1)) / dz_;
      dwdz = (U(i, j, k + 1, 2) - U(i, j, k, 2)) / dz_;
    }
    STR(i, j, k, 0) = (2.0 / 3.0) * mu * (2.0 * dudx - dvdy - dwdz);
    STR(i, j, k, 1) = (2.0 / 3.0) * mu * (2.0 * dvdy - dudx - dwdz);
    STR(i, j, k, 2) = (2.0 / 3.0) * mu * (2.0 * dwdz - dudx - dvdy);
    STR(i, j, k, 3) = mu * (dudy + dvdx);
    STR(i, j, k, 4) = mu * (dudz + dwdx);
    STR(i, j, k, 5) = mu * (dvdz + dwdy);
  }
  // applyViscousTerm{x,y,z}3dv (src/viscosity.hpp:460-498, 542-580, 625-663)
  void applyVisc3D(int dir, int i, int j, int k) {
    const int ih = dir == 0, jh = dir == 1, kh = dir == 2;
    const double d = dir == 0 ? cd[1] : dir == 1 ? cd[2] : cd[3];
    // stress components carried by the momenta / energy on this face set
    static const int comp[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
    const int* c = comp[dir];
    double ur = (VEL(i + ih, j + jh, k + kh, 0) + VEL(i, j, k, 0)) / 2.0;
    double ul = (VEL(i - ih, j - jh, k - kh, 0) + VEL(i, j, k, 0)) / 2.0;
    double vr = (VEL(i + ih, j + jh, k + kh, 1) + VEL(i, j, k, 1)) / 2.0;
    double vl = (VEL(i - ih, j - jh, k - kh, 1) + VEL(i, j, k, 1)) / 2.0;
    double wr = (VEL(i + ih, j + jh, k + kh, 2) + VEL(i, j, k, 2)) / 2.0;
    double wl = (VEL(i - ih, j - jh, k - kh, 2) + VEL(i, j, k, 2)) / 2.0;
    auto S = [&](int a, int b, int cc, int n) { return STR(a, b, cc, n); };
    int im = i - ih, jm = j - jh, km = k - kh;
    double a = (S(i, j, k, c[0]) - S(im, jm, km, c[0])) / d;
    double b = (S(i, j, k, c[1]) - S(im, jm, km, c[1])) / d;
    double cc = (S(i, j, k, c[2]) - S(im, jm, km, c[2])) / d;
    // energy: u-weighted term uses the x-momentum component of this face
    // set first, then y, then z (src/viscosity.hpp:488-490, 570-572, 653-655)
    double dd = (ur * S(i, j, k, c[0]) - ul * S(im, jm, km, c[0])) / d +
                (vr * S(i, j, k, c[1]) - vl * S(im, jm, km, c[1])) / d +
                (wr * S(i, j, k, c[2]) - wl * S(im, jm, km, c[2])) / d;
    D(i, j, k, 0) += a;
    D(i, j, k, 1) += b;
    D(i, j, k, 2) += cc;
    D(i, j, k, 3) += dd;
  }
  // calculateRhoGrad (src/ceq3d.hpp:95-187)
  double nrg3(int i, int j, int k) {
    return V(i, j, k, 3) / RHO(i, j, k) -
           0.5 * RHO(i, j, k) * (VEL(i, j, k, 0) * VEL(i, j, k, 0) + VEL(i, j, k, 1) * VEL(i, j, k, 1) +
                                 VEL(i, j, k, 2) * VEL(i, j, k, 2));
  }
  void rhoGrad3D(int i, int j, int k) {
    auto dR = [&](int ih, int jh, int kh, double d) {
      return (RHO(i - 2 * ih, j - 2 * jh, k - 2 * kh) - 8.0 * RHO(i - ih, j - jh, k - kh) +
              8.0 * RHO(i + ih, j + jh, k + kh) - RHO(i + 2 * ih, j + 2 * jh, k + 2 * kh)) / (12.0 * d);
    };
    auto dE = [&](int ih, int jh, int kh, double d) {
      return (nrg3(i - 2 * ih, j - 2 * jh, k - 2 * kh) - 8.0 * nrg3(i - ih, j - jh, k - kh) +
              8.0 * nrg3(i + ih, j + jh, k + kh) - nrg3(i + 2 * ih, j + 2 * jh, k + 2 * kh)) / (12.0 * d);
    };
    auto dU = [&](int ih, int jh, int kh, int v, double d) {
      return (VEL(i - 2 * ih, j - 2 * jh, k - 2 * kh, v) - 8.0 * VEL(i - ih, j - jh, k - kh, v) +
              8.0 * VEL(i + ih, j + jh, k + kh, v) - VEL(i + 2 * ih, j + 2 * jh, k + 2 * kh, v)) / (12.0 * d);
    };
    double dxr = dR(1, 0, 0, dx), dyr = dR(0, 1, 0, dy), dzr = dR(0, 0, 1, dz);
    double dxe = dE(1, 0, 0, dx), dye = dE(0, 1, 0, dy), dze = dE(0, 0, 1, dz);
    double dxu = dU(1, 0, 0, 0, dx), dyv = dU(0, 1, 0, 1, dy), dzw = dU(0, 0, 1, 2, dz);
    double n1 = dxr, n2 = dyr, n3 = dzr;
    double rgrad = std::sqrt(dxr * dxr + dyr * dyr + dzr * dzr);
    double divu = dxu + dyv + dzw;
    double dnednr = (n1 * dxe + n2 * dye + n3 * dze) * (n1 * dxr + n2 * dyr + n3 * dzr);
    int indicator = dnednr < 0.0 ? 1 : 0;
    if (divu < 0) GR(i, j, k, 0) = (1 - indicator) * rgrad;
    else GR(i, j, k, 0) = 0;
    GR(i, j, k, 1) = indicator * rgrad;
    GR(i, j, k, 2) = dxr;
    GR(i, j, k, 3) = dyr;
    GR(i, j, k, 4) = dzr;
  }
  // maxWaveSpeed (src/ceq3d.hpp:25-63)
  double waveSpeed3D(int i, int j, int k) {
    double gamma, gammas, Rs, Cp = 0, Cv = 0, a, s;
    for (int sp = 0; sp < ns; ++sp) {
      gammas = cd[6 + 3 * sp];
      Rs = cd[6 + 3 * sp + 1];
      Cp = Cp + (V(i, j, k, 4 + sp) / RHO(i, j, k)) * (gammas * Rs / (gammas - 1));
      Cv = Cv + (V(i, j, k, 4 + sp) / RHO(i, j, k)) * (Rs / (gammas - 1));
    }
    gamma = Cp / Cv;
    a = std::sqrt(gamma * P(i, j, k) / RHO(i, j, k));
    s = a + std::sqrt(V(i, j, k, 0) * V(i, j, k, 0) + V(i, j, k, 1) * V(i, j, k, 1) +
                      V(i, j, k, 2) * V(i, j, k, 2)) / RHO(i, j, k);
    return s;
  }
  // updateCeq (src/ceq3d.hpp:189-224)
  void updateCeq3D(int i, int j, int k, double maxS) {
    double dx_ = cd[1], dy_ = cd[2], dz_ = cd[3];
    int nc = (int)cd[0] + 4;
    double dxm = std::sqrt(dx_ * dx_ + dy_ * dy_ + dz_ * dz_);
    for (int n = 0; n < 5; ++n) {
      double lap = (V(i - 1, j, k, nc + n) - 2 * V(i, j, k, nc + n) + V(i + 1, j, k, nc + n)) / dx_ +
                   (V(i, j - 1, k, nc + n) - 2 * V(i, j, k, nc + n) + V(i, j + 1, k, nc + n)) / dy_ +
                   (V(i, j, k - 1, nc + n) - 2 * V(i, j, k, nc + n) + V(i, j, k + 1, nc + n)) / dz_;
      D(i, j, k, nc + n) = (maxS / (cf.eps * dxm)) * (GR(i, j, k, n) - V(i, j, k, nc + n)) +
                           cf.kap * maxS * dxm * lap;
    }
  }
  // calculateCeqFaces (src/ceq3d.hpp:226-296)
  void ceqFaces3D(int i, int j, int k, double alpha) {
    for (int face = 0; face < 3; ++face) {
      int ip = face == 0, jp = face == 1, kp = face == 2;
      double r = (RHO(i, j, k) + RHO(i + ip, j + jp, k + kp)) / 2.0;
      auto iC = [&](int v) { return (V(i, j, k, nv + v) + V(i + ip, j + jp, k + kp, nv + v)) / 2.0; };
      double chat = iC(1);
      double cn[3] = {iC(2), iC(3), iC(4)};
      double cmag = 1.0e-6;
      cmag += cn[0] * cn[0];
      cmag += cn[1] * cn[1];
      cmag += cn[2] * cn[2];
      for (int dir = 0; dir < 3; ++dir) {
        double dirac = face == dir ? 1.0 : 0.0;
        double M = dirac - (cn[face] * cn[dir]) / cmag;
        for (int w = 0; w < 3; ++w) MF3(face, dir, i, j, k, w) = alpha * r * chat * M;
      }
    }
  }
  // calculateCeqGrads (src/ceq3d.hpp:298-332)
  void ceqGrads3D(int i, int j, int k) {
    auto U = [&](int a, int b, int c, int w) { return VEL(a, b, c, w); };
    for (int w = 0; w < 3; ++w) {
      MF3(0, 0, i, j, k, w) *= (U(i + 1, j, k, w) - U(i, j, k, w)) / dx;
      MF3(0, 1, i, j, k, w) *= ((U(i, j + 1, k, w) + U(i + 1, j + 1, k, w)) - (U(i, j - 1, k, w) + U(i + 1, j - 1, k, w))) / (4 * dy);
      MF3(0, 2, i, j, k, w) *= ((U(i, j, k + 1, w) + U(i + 1, j, k + 1, w)) - (U(i, j, k - 1, w) + U(i + 1, j, k - 1, w))) / (4 * dz);
      MF3(1, 0, i, j, k, w) *= ((U(i + 1, j + 1, k, w) + U(i + 1, j, k, w)) - (U(i - 1, j + 1, k, w) + U(i - 1, j, k, w))) / (4 * dx);
      MF3(1, 1, i, j, k, w) *= (U(i, j + 1, k, w) - U(i, j, k, w)) / dy;
      MF3(1, 2, i, j, k, w) *= ((U(i, j + 1, k + 1, w) + U(i, j, k + 1, w)) - (U(i, j + 1, k - 1, w) + U(i, j, k - 1, w))) / (4 * dz);
      MF3(2, 0, i, j, k, w) *= ((U(i + 1, j, k + 1, w) + U(i + 1, j, k, w)) - (U(i - 1, j, k + 1, w) + U(i - 1, j, k, w))) / (4 * dx);
      MF3(2, 1, i, j, k, w) *= ((U(i, j + 1, k + 1, w) + U(i, j + 1, k, w)) - (U(i, j - 1, k + 1, w) + U(i, j - 1, k, w))) / (4 * dy);
      MF3(2, 2, i, j, k, w) *= (U(i, j, k + 1, w) - U(i, j, k, w)) / dz;
    }
  }
  // applyCeq (src/ceq3d.hpp:334-366)
  void applyCeq3D(int i, int j, int k) {
    const double d[3] = {dx, dy, dz};
    for (int w = 0; w < 3; ++w) {
      double diffu = 0.0;
      for (int face = 0; face < 3; ++face) {
        int ih = face == 0, jh = face == 1, kh = face == 2;
        for (int dir = 0; dir < 3; ++dir)
          diffu += (MF3(face, dir, i, j, k, w) - MF3(face, dir, i - ih, j - jh, k - kh, w)) / d[face];
      }
      D(i, j, k, w) += diffu;
    }
  }

  // cart3d_func::compute (src/cart3d.cpp:220-298)
  void compute3D() {
    apply_bcs();
    const int b = ng, ei = ngi - ng, ej = ngj - ng, ek = ngk - ng;
    box(0, ngi, 0, ngj, 0, ngk, [&](int i, int j, int k) { rhoPT3D(i, j, k); });
    box(0, ngi, 0, ngj, 0, ngk, [&](int i, int j, int k) { velocity3D(i, j, k); });
    for (int v = 0; v < nv; ++v) {
      box(b - 1, ei, b - 1, ej, b - 1, ek, [&](int i, int j, int k) { fluxes3D(i, j, k, v); });
      box(b, ei, b, ej, b, ek, [&](int i, int j, int k) { advect3D(i, j, k, v); });
    }
    box(b, ei, b, ej, b, ek, [&](int i, int j, int k) { presgrad3D(i, j, k); });
    if (cf.buoyancy) box(b, ei, b, ej, b, ek, [&](int i, int j, int k) { buoyancy3D(i, j, k); });
    if (cf.visc) {
      for (int dir = 0; dir < 3; ++dir) {
        box(b - 1, ei, b - 1, ej, b - 1, ek, [&](int i, int j, int k) { stress3D(dir, i, j, k); });
        box(b, ei, b, ej, b, ek, [&](int i, int j, int k) { applyVisc3D(dir, i, j, k); });
      }
    }
    if (cf.ceq) {
      box(b, ei, b, ej, b, ek, [&](int i, int j, int k) { rhoGrad3D(i, j, k); });
      double maxS = box_max(b, ei, b, ej, b, ek, [&](int i, int j, int k) { return waveSpeed3D(i, j, k); });
      // maxGradFunctor(var, nv+1): |C_hat| read from var (src/ceq3d.hpp:82-93, src/cart3d.cpp:283)
      double maxCh = box_max(b, ei, b, ej, b, ek, [&](int i, int j, int k) { return std::fabs(V(i, j, k, nv + 1)); });
      double alpha = (dxmag / (maxCh + 1.0e-6)) * cf.alpha;
      last_maxS = maxS;
      last_maxCh = maxCh;
      box(b, ei, b, ej, b, ek, [&](int i, int j, int k) { updateCeq3D(i, j, k, maxS); });
      box(b - 1, ei, b - 1, ej, b - 1, ek, [&](int i, int j, int k) { ceqFaces3D(i, j, k, alpha); });
      box(b - 1, ei, b - 1, ej, b - 1, ek, [&](int i, int j, int k) { ceqGrads3D(i, j, k); });
      box(b, ei, b, ej, b, ek, [&](int i, int j, int k) { applyCeq3D(i, j, k); });
    }
  }

  // ==================================================================
  // 2D kernels
  // ==================================================================
  // calculateRhoPT2D (src/secondary.hpp:60-107)
  void rhoPT2D(int i, int j) {
    double gamma, gammas, Rs, Cp = 0, Cv = 0;
    RHO(i, j, 0) = 0.0;
    for (int s = 0; s < ns; ++s) RHO(i, j, 0) = RHO(i, j, 0) + V(i, j, 0, 3 + s);
    for (int s = 0; s < ns; ++s) {
      gammas = cd[6 + 3 * s];
      Rs = cd[6 + 3 * s + 1];
      Cp = Cp + (V(i, j, 0, 3 + s) / RHO(i, j, 0)) * (gammas * Rs / (gammas - 1));
      Cv = Cv + (V(i, j, 0, 3 + s) / RHO(i, j, 0)) * (Rs / (gammas - 1));
    }
    gamma = Cp / Cv;
    P(i, j, 0) = (gamma - 1) * (V(i, j, 0, 2) - (0.5 / RHO(i, j, 0)) *
                                                    (V(i, j, 0, 0) * V(i, j, 0, 0) + V(i, j, 0, 1) * V(i, j, 0, 1)));
    TT(i, j, 0) = P(i, j, 0) / ((Cp - Cv) * RHO(i, j, 0));
  }
  // computeVelocity2D (src/velocity.hpp:85-99)
  void velocity2D(int i, int j) {
    VEL(i, j, 0, 0) = V(i, j, 0, 0) / RHO(i, j, 0);
    VEL(i, j, 0, 1) = V(i, j, 0, 1) / RHO(i, j, 0);
  }
  // computeFluxWeno2D::weno (src/flux.hpp:37-63): double constants.
  static inline double weno2(double f1, double f2, double f3, double f4, double f5) {
    const double eps = 1e-6;
    double b1, b2, b3, w1, w2, w3, p1, p2, p3, a1, a2;
    a1 = f1 - 2.0 * f2 + f3;
    a2 = f1 - 4.0 * f2 + 3.0 * f3;
    b1 = (13.0 / 12.0) * a1 * a1 + (0.25) * a2 * a2;
    a1 = f2 - 2.0 * f3 + f4;
    a2 = f2 - f4;
    b2 = (13.0 / 12.0) * a1 * a1 + (0.25) * a2 * a2;
    a1 = f3 - 2.0 * f4 + f5;
    a2 = 3.0 * f3 - 4.0 * f4 + f5;
    b3 = (13.0 / 12.0) * a1 * a1 + (0.25) * a2 * a2;
    a1 = eps + b1;
    w1 = (0.1) / (a1 * a1);
    a1 = eps + b2;
    w2 = (0.6) / (a1 * a1);
    a1 = eps + b3;
    w3 = (0.3) / (a1 * a1);
    p1 = (1.0 / 3.0) * f1 + (-7.0 / 6.0) * f2 + (11.0 / 6.0) * f3;
    p2 = (-1.0 / 6.0) * f2 + (5.0 / 6.0) * f3 + (1.0 / 3.0) * f4;
    p3 = (1.0 / 3.0) * f3 + (5.0 / 6.0) * f4 + (-1.0 / 6.0) * f5;
    return (w1 * p1 + w2 * p2 + w3 * p3) / (w1 + w2 + w3);
  }
  // computeFluxWeno2D::operator() (src/flux.hpp:65-105)
  void fluxes2D(int i, int j, int v) {
    double ur, vr, f1, f2, f3, f4, f5;
    auto q = [&](int a, int b) { return V(a, b, 0, v) + (v == 2) * P(a, b, 0); };
    ur = (-VEL(i + 2, j, 0, 0) + 7.0 * VEL(i + 1, j, 0, 0) + 7.0 * VEL(i, j, 0, 0) - VEL(i - 1, j, 0, 0)) / 12.0;
    vr = (-VEL(i, j + 2, 0, 1) + 7.0 * VEL(i, j + 1, 0, 1) + 7.0 * VEL(i, j, 0, 1) - VEL(i, j - 1, 0, 1)) / 12.0;
    if (ur < 0.0) { f1 = q(i + 3, j); f2 = q(i + 2, j); f3 = q(i + 1, j); f4 = q(i, j); f5 = q(i - 1, j); }
    else          { f1 = q(i - 2, j); f2 = q(i - 1, j); f3 = q(i, j); f4 = q(i + 1, j); f5 = q(i + 2, j); }
    fluxx[c3(i, j, 0)] = ur * weno2(f1, f2, f3, f4, f5) / dx;
    if (vr < 0.0) { f1 = q(i, j + 3); f2 = q(i, j + 2); f3 = q(i, j + 1); f4 = q(i, j); f5 = q(i, j - 1); }
    else          { f1 = q(i, j - 2); f2 = q(i, j - 1); f3 = q(i, j); f4 = q(i, j + 1); f5 = q(i, j + 2); }
    fluxy[c3(i, j, 0)] = vr * weno2(f1, f2, f3, f4, f5) / dy;
  }
  // advect2D (src/advect.hpp:23-37)
  void advect2D(int i, int j, int v) {
    D(i, j, 0, v) = -((fluxx[c3(i, j, 0)] - fluxx[c3(i - 1, j, 0)]) + (fluxy[c3(i, j, 0)] - fluxy[c3(i, j - 1, 0)]));
  }
  // applyPressureGradient2D (src/presgrad.hpp:21-42)
  void presgrad2D(int i, int j) {
    double dx_ = cd[1], dy_ = cd[2];
    double dxp = (P(i - 2, j, 0) - 8.0 * P(i - 1, j, 0) + 8.0 * P(i + 1, j, 0) - P(i + 2, j, 0)) / (12.0 * dx_);
    double dyp = (P(i, j - 2, 0) - 8.0 * P(i, j - 1, 0) + 8.0 * P(i, j + 1, 0) - P(i, j + 2, 0)) / (12.0 * dy_);
    D(i, j, 0, 0) -= dxp;
    D(i, j, 0, 1) -= dyp;
  }
  // computeBuoyancy (src/buoyancy.hpp:49-73)
  void buoyancy2D(int i, int j) {
    double vv = V(i, j, 0, 1) / V(i, j, 0, 3);
    double rhop = RHO(i, j, 0) - cf.rho_ref;
    double eps = 1e-6;
    if (rhop >= eps || rhop <= -eps) {
      double f = -cf.g_accel * rhop;
      D(i, j, 0, 1) += f;
      D(i, j, 0, 2) += std::fabs(vv) * f;
    }
  }
  // calculateStressTensor2dv (src/viscosity.hpp:25-109): constant mu, and
  // the reference's vel(i,j-1,1) in the x-face dudy.
  void stress2D(int i, int j) {
    double dx_ = cd[1], dy_ = cd[2];
    double dudx, dvdy, dudy, dvdx;
    double mur = 2.928e-5, mut = 2.928e-5;
    auto U = [&](int a, int b, int d) { return VEL(a, b, 0, d); };
    dudx = (U(i + 1, j, 0) - U(i, j, 0)) / dx_;
    dvdx = (U(i + 1, j, 1) - U(i, j, 1)) / dx_;
    dudy = ((U(i, j + 1, 0) + U(i + 1, j + 1, 0)) - (U(i, j - 1, 1) + U(i + 1, j - 1, 0))) / (4.0 * dy_);
    dvdy = ((U(i, j + 1, 1) + U(i + 1, j + 1, 1)) - (U(i, j - 1, 1) + U(i + 1, j - 1, 1))) / (4.0 * dy_);
    SX(i, j, 0, 0) = (2.0 / 3.0) * mur * (2.0 * dudx - dvdy);
    SX(i, j, 1, 1) = (2.0 / 3.0) * mur * (2.0 * dvdy - dudx);
    SX(i, j, 0, 1) = mur * (dudy + dvdx);
    SX(i, j, 1, 0) = SX(i, j, 0, 1);
    dudx = ((U(i + 1, j, 0) + U(i + 1, j + 1, 0)) - (U(i - 1, j, 0) + U(i - 1, j + 1, 0))) / (4.0 * dx_);
    dvdx = ((U(i + 1, j, 1) + U(i + 1, j + 1, 1)) - (U(i - 1, j, 1) + U(i - 1, j + 1, 1))) / (4.0 * dx_);
    dudy = (U(i, j + 1, 0) - U(i, j, 0)) / dy_;
    dvdy = (U(i, j + 1, 1) - U(i, j, 1)) / dy_;
    SY(i, j, 0, 0) = (2.0 / 3.0) * mut * (2.0 * dudx - dvdy);
    SY(i, j, 1, 1) = (2.0 / 3.0) * mut * (2.0 * dvdy - dudx);
    SY(i, j, 0, 1) = mut * (dudy + dvdx);
    SY(i, j, 1, 0) = SY(i, j, 0, 1);
  }
  // calculateHeatFlux2dv (src/viscosity.hpp:111-136), k = 0.026
  void heatflux2D(int i, int j) {
    const double kk = 0.026;
    QX(i, j) = -kk * (TT(i + 1, j, 0) - TT(i, j, 0)) / cd[1];
    QY(i, j) = -kk * (TT(i, j + 1, 0) - TT(i, j, 0)) / cd[2];
  }
  // applyViscousTerm2dv (src/viscosity.hpp:138-199)
  void applyVisc2D(int i, int j) {
    double dx_ = cd[1], dy_ = cd[2];
    auto U = [&](int a, int b, int d) { return VEL(a, b, 0, d); };
    double ur = (U(i + 1, j, 0) + U(i, j, 0)) / 2.0;
    double ul = (U(i - 1, j, 0) + U(i, j, 0)) / 2.0;
    double vr = (U(i + 1, j, 1) + U(i, j, 1)) / 2.0;
    double vl = (U(i - 1, j, 1) + U(i, j, 1)) / 2.0;
    double ut = (U(i, j + 1, 0) + U(i, j, 0)) / 2.0;
    double ub = (U(i, j - 1, 0) + U(i, j, 0)) / 2.0;
    double vt = (U(i, j + 1, 1) + U(i, j, 1)) / 2.0;
    double vb = (U(i, j - 1, 1) + U(i, j, 1)) / 2.0;
    double a = (SX(i, j, 0, 0) - SX(i - 1, j, 0, 0)) / dx_ + (SY(i, j, 0, 1) - SY(i, j - 1, 0, 1)) / dy_;
    double b = (SX(i, j, 1, 0) - SX(i - 1, j, 1, 0)) / dx_ + (SY(i, j, 1, 1) - SY(i, j - 1, 1, 1)) / dy_;
    double c1 = (ur * SX(i, j, 0, 0) - ul * SX(i - 1, j, 0, 0)) / dx_ +
                (vr * SX(i, j, 0, 1) - vl * SX(i - 1, j, 0, 1)) / dx_ +
                (ut * SY(i, j, 1, 0) - ub * SY(i, j - 1, 1, 0)) / dy_ +
                (vt * SY(i, j, 1, 1) - vb * SY(i, j - 1, 1, 1)) / dy_;
    double c2 = (QX(i, j) - QX(i - 1, j)) / dx_ + (QY(i, j) - QY(i, j - 1)) / dy_;
    D(i, j, 0, 0) = D(i, j, 0, 0) + a;
    D(i, j, 0, 1) = D(i, j, 0, 1) + b;
    D(i, j, 0, 2) = D(i, j, 0, 2) + c1 - c2;
  }
  // calculateRhoGrad2D (src/ceq.hpp:80-152)
  double nrg2(int i, int j) {
    return V(i, j, 0, 2) / RHO(i, j, 0) -
           0.5 * RHO(i, j, 0) * (VEL(i, j, 0, 0) * VEL(i, j, 0, 0) + VEL(i, j, 0, 1) * VEL(i, j, 0, 1));
  }
  void rhoGrad2D(int i, int j) {
    auto dR = [&](int ih, int jh, double d) {
      return (RHO(i - 2 * ih, j - 2 * jh, 0) - 8.0 * RHO(i - ih, j - jh, 0) + 8.0 * RHO(i + ih, j + jh, 0) -
              RHO(i + 2 * ih, j + 2 * jh, 0)) / (12.0 * d);
    };
    auto dE = [&](int ih, int jh, double d) {
      return (nrg2(i - 2 * ih, j - 2 * jh) - 8.0 * nrg2(i - ih, j - jh) + 8.0 * nrg2(i + ih, j + jh) -
              nrg2(i + 2 * ih, j + 2 * jh)) / (12.0 * d);
    };
    auto dU = [&](int ih, int jh, int v, double d) {
      return (VEL(i - 2 * ih, j - 2 * jh, 0, v) - 8.0 * VEL(i - ih, j - jh, 0, v) + 8.0 * VEL(i + ih, j + jh, 0, v) -
              VEL(i + 2 * ih, j + 2 * jh, 0, v)) / (12.0 * d);
    };
    double dxr = dR(1, 0, dx), dyr = dR(0, 1, dy);
    double dxe = dE(1, 0, dx), dye = dE(0, 1, dy);
    double dxu = dU(1, 0, 0, dx), dyv = dU(0, 1, 1, dy);
    double n1 = dxr, n2 = dyr;
    double rgrad = std::sqrt(dxr * dxr + dyr * dyr);
    double divu = dxu + dyv;
    double dnednr = (n1 * dxe + n2 * dye) * (n1 * dxr + n2 * dyr);
    double i1 = dnednr < 0.0 ? 1.0 : 0.0;
    double i2 = 0;
    if (divu < 0.0) i2 = 1.0;
    GR(i, j, 0, 0) = (1 - i1) * i2 * rgrad;
    GR(i, j, 0, 1) = i1 * rgrad;
    GR(i, j, 0, 2) = -dyr;
    GR(i, j, 0, 3) = dxr;
  }
  // maxWaveSpeed2D (src/ceq.hpp:42-78): species stride 2 and no /rho on the
  // momentum magnitude, as the reference has them.
  double waveSpeed2D(int i, int j) {
    double gamma, gammas, Rs, Cp = 0, Cv = 0, a, s;
    for (int sp = 0; sp < ns; ++sp) {
      gammas = cd[6 + 2 * sp];
      Rs = cd[6 + 2 * sp + 1];
      Cp = Cp + (V(i, j, 0, 3 + sp) / RHO(i, j, 0)) * (gammas * Rs / (gammas - 1));
      Cv = Cv + (V(i, j, 0, 3 + sp) / RHO(i, j, 0)) * (Rs / (gammas - 1));
    }
    gamma = Cp / Cv;
    a = std::sqrt(gamma * P(i, j, 0) / RHO(i, j, 0));
    s = a + std::sqrt(V(i, j, 0, 0) * V(i, j, 0, 0) + V(i, j, 0, 1) * V(i, j, 0, 1));
    return s;
  }
  // updateCeq2D (src/ceq.hpp:154-198)
  void updateCeq2D(int i, int j, double maxS) {
    double dx_ = cd[1], dy_ = cd[2];
    int nc = (int)cd[0] + 3;
    double dxm = std::sqrt(dx_ * dx_ + dy_ * dy_);
    for (int n = 0; n < 4; ++n) {
      double dx_right = (V(i + 1, j, 0, nc + n) - V(i, j, 0, nc + n)) / dx_;
      double dx_left = (V(i, j, 0, nc + n) - V(i - 1, j, 0, nc + n)) / dx_;
      double dy_top = (V(i, j + 1, 0, nc + n) - V(i, j, 0, nc + n)) / dy_;
      double dy_bot = (V(i, j, 0, nc + n) - V(i, j - 1, 0, nc + n)) / dy_;
      double lap = dx_right - dx_left + dy_top - dy_bot;
      D(i, j, 0, nc + n) = (maxS / (cf.eps * dxm)) * (GR(i, j, 0, n) - V(i, j, 0, nc + n)) + cf.kap * maxS * dxm * lap;
    }
  }
  // computeCeqFlux2D (src/ceq.hpp:200-245)
  void ceqFlux2D(int i, int j, double alpha) {
    for (int f = 0; f < 2; ++f) {
      int ih = f == 0, jh = f == 1;
      double r = (RHO(i, j, 0) + RHO(i + ih, j + jh, 0)) / 2.0;
      auto iC = [&](int v) { return (V(i, j, 0, nv + v) + V(i + ih, j + jh, 0, nv + v)) / 2.0; };
      double chat = iC(1);
      double ct[2] = {iC(2), iC(3)};
      double ctmag = (ct[0] * ct[0] + ct[1] * ct[1]) + 1.0e-6;
      for (int d = 0; d < 2; ++d)
        for (int w = 0; w < 2; ++w) M2(f, d, i, j, w) = alpha * r * chat * (ct[f] * ct[d]) / ctmag;
    }
  }
  // computeCeqFaces2D (src/ceq.hpp:247-267)
  void ceqFaces2D(int i, int j) {
    auto U = [&](int a, int b, int w) { return VEL(a, b, 0, w); };
    for (int w = 0; w < 2; ++w) {
      M2(0, 0, i, j, w) *= (U(i + 1, j, w) - U(i, j, w)) / dx;
      M2(0, 1, i, j, w) *= ((U(i, j + 1, w) + U(i + 1, j + 1, w)) - (U(i, j - 1, w) + U(i + 1, j - 1, w))) / (4.0 * dy);
      M2(1, 0, i, j, w) *= ((U(i + 1, j, w) + U(i + 1, j + 1, w)) - (U(i - 1, j, w) + U(i - 1, j + 1, w))) / (4.0 * dx);
      M2(1, 1, i, j, w) *= (U(i, j + 1, w) - U(i, j, w)) / dy;
    }
  }
  // applyCeq2D (src/ceq.hpp:269-291)
  void applyCeq2D(int i, int j) {
    for (int w = 0; w < 2; ++w) {
      double diffu = 0;
      diffu += (M2(0, 0, i, j, w) - M2(0, 0, i - 1, j, w)) / dx;
      diffu += (M2(0, 1, i, j, w) - M2(0, 1, i - 1, j, w)) / dx;
      diffu += (M2(1, 0, i, j, w) - M2(1, 0, i, j - 1, w)) / dy;
      diffu += (M2(1, 1, i, j, w) - M2(1, 1, i, j - 1, w)) / dy;
      D(i, j, 0, w) += diffu;
    }
  }

  // cart2d_func::compute (src/cart2d.cpp:151-237); BCs are in preStep.
  void compute2D() {
    const int b = ng, ei = ngi - ng, ej = ngj - ng;
    box(0, ngi, 0, ngj, 0, 1, [&](int i, int j, int) { rhoPT2D(i, j); });
    box(0, ngi, 0, ngj, 0, 1, [&](int i, int j, int) { velocity2D(i, j); });
    for (int v = 0; v < nv; ++v) {
      box(b - 1, ei, b - 1, ej, 0, 1, [&](int i, int j, int) { flux2D_any(i, j, v); });
      box(b, ei, b, ej, 0, 1, [&](int i, int j, int) { advect2D(i, j, v); });
    }
    box(b, ei, b, ej, 0, 1, [&](int i, int j, int) { presgrad2D(i, j); });
    if (cf.buoyancy) box(b, ei, b, ej, 0, 1, [&](int i, int j, int) { buoyancy2D(i, j); });
    if (cf.visc) {
      box(b - 1, ei, b - 1, ej, 0, 1, [&](int i, int j, int) { stress2D(i, j); });
      box(b - 1, ei, b - 1, ej, 0, 1, [&](int i, int j, int) { heatflux2D(i, j); });
      box(b, ei, b, ej, 0, 1, [&](int i, int j, int) { applyVisc2D(i, j); });
    }
    if (cf.ceq) {
      box(b, ei, b, ej, 0, 1, [&](int i, int j, int) { rhoGrad2D(i, j); });
      double maxS = box_max(b, ei, b, ej, 0, 1, [&](int i, int j, int) { return waveSpeed2D(i, j); });
      double maxCh = box_max(b, ei, b, ej, 0, 1, [&](int i, int j, int) { return std::fabs(V(i, j, 0, nv + 1)); });
      double alpha = (dx * dx + dy * dy) / (maxCh + 1.0e-6) * cf.alpha;
      last_maxS = maxS;
      last_maxCh = maxCh;
      box(b, ei, b, ej, 0, 1, [&](int i, int j, int) { updateCeq2D(i, j, maxS); });
      box(b - 1, ei, b - 1, ej, 0, 1, [&](int i, int j, int) { ceqFlux2D(i, j, alpha); });
      box(b - 1, ei, b - 1, ej, 0, 1, [&](int i, int j, int) { ceqFaces2D(i, j); });
      box(b, ei, b, ej, 0, 1, [&](int i, int j, int) { applyCeq2D(i, j); });
    }
  }

  // ==================================================================
  // 2D centred and QUICK fluxes (cf.scheme 2 and 3), src/flux.hpp:108-221
  // ==================================================================
  // computeFluxCentered2D::operator() (src/flux.hpp:121-166)
  void fluxCentered2D(int i, int j, int v) {
    double ur, vr, x1, y1, px, py;
    ur = (0.0 - V(i + 2, j, 0, 0) / RHO(i + 2, j, 0) + 7.0 * V(i + 1, j, 0, 0) / RHO(i + 1, j, 0) +
          7.0 * V(i, j, 0, 0) / RHO(i, j, 0) - V(i - 1, j, 0, 0) / RHO(i - 1, j, 0)) / 12.0;
    vr = (0.0 - V(i, j + 2, 0, 1) / RHO(i, j + 2, 0) + 7.0 * V(i, j + 1, 0, 1) / RHO(i, j + 1, 0) +
          7.0 * V(i, j, 0, 1) / RHO(i, j, 0) - V(i, j - 1, 0, 1) / RHO(i, j - 1, 0)) / 12.0;
    px = (0.0 - P(i + 2, j, 0) + 7.0 * P(i + 1, j, 0) + 7.0 * P(i, j, 0) - P(i - 1, j, 0)) / 12.0;
    py = (0.0 - P(i, j + 2, 0) + 7.0 * P(i, j + 1, 0) + 7.0 * P(i, j, 0) - P(i, j - 1, 0)) / 12.0;
    x1 = (0.0 - V(i + 2, j, 0, v) + 7.0 * V(i + 1, j, 0, v) + 7.0 * V(i, j, 0, v) - V(i - 1, j, 0, v)) / 12.0;
    y1 = (0.0 - V(i, j + 2, 0, v) + 7.0 * V(i, j + 1, 0, v) + 7.0 * V(i, j, 0, v) - V(i, j - 1, 0, v)) / 12.0;
    if (v == 2) {
      x1 = x1 + px;
      y1 = y1 + py;
    }
    fluxx[c3(i, j, 0)] = ur * x1 / cd[1];
    fluxy[c3(i, j, 0)] = vr * y1 / cd[2];
  }
  // computeFluxQuick2D::operator() (src/flux.hpp:187-220)
  void fluxQuick2D(int i, int j, int v) {
    auto q = [&](int a, int b) { return V(a, b, 0, v) + (v == 2) * P(a, b, 0); };
    auto quick = [](double f1, double f2, double f3) { return 0.75 * f2 + 0.375 * f3 - 0.125 * f1; };
    double ur = (-VEL(i + 2, j, 0, 0) + 7.0 * VEL(i + 1, j, 0, 0) + 7.0 * VEL(i, j, 0, 0) - VEL(i - 1, j, 0, 0)) / 12.0;
    double f1, f2, f3;
    if (ur < 0.0) { f1 = q(i + 2, j); f2 = q(i + 1, j); f3 = q(i, j); }
    else          { f1 = q(i - 1, j); f2 = q(i, j); f3 = q(i + 1, j); }
    fluxx[c3(i, j, 0)] = ur * quick(f1, f2, f3) / cd[1];
    double vr = (-VEL(i, j + 2, 0, 1) + 7.0 * VEL(i, j + 1, 0, 1) + 7.0 * VEL(i, j, 0, 1) - VEL(i, j - 1, 0, 1)) / 12.0;
    if (vr < 0.0) { f1 = q(i, j + 2); f2 = q(i, j + 1); f3 = q(i, j); }
    else          { f1 = q(i, j - 1); f2 = q(i, j); f3 = q(i, j + 1); }
    fluxy[c3(i, j, 0)] = vr * quick(f1, f2, f3) / cd[2];
  }
  void flux2D_any(int i, int j, int v) {
    if (scheme == 3) fluxQuick2D(i, j, v);
    else if (scheme == 2) fluxCentered2D(i, j, v);
    else fluxes2D(i, j, v);
  }

  // ==================================================================
  // Generalized grids: src/metric.hpp, src/gen3d.cpp, src/gen2d.cpp
  // ==================================================================
  inline double X(int ii, int jj, int kk, int d) const {
    return nodes[(size_t)ii + (size_t)ni * (jj + (size_t)nj * (kk + (size_t)nk * d))];
  }
  inline double& MT(int i, int j, int k, int a, int b) {
    return met[(c3(i, j, k) * ndim + a) * ndim + b];
  }
  // computeMetrics3D::operator() (src/metric.hpp:62-164), written out term by term
  void metrics3D(int i, int j, int k) {
    const int a = i - 3, b = j - 3, c = k - 3;
    double fm[3][3], fp[3][3];  // [face axis][component]: centroid of the - / + face
    for (int d = 0; d < 3; ++d) {
      fm[0][d] = (X(a, b, c, d) + X(a, b + 1, c, d) + X(a, b, c + 1, d) + X(a, b + 1, c + 1, d)) / 4.0;
      fp[0][d] = (X(a + 1, b, c, d) + X(a + 1, b + 1, c, d) + X(a + 1, b, c + 1, d) + X(a + 1, b + 1, c + 1, d)) / 4.0;
      fm[2][d] = (X(a, b, c, d) + X(a + 1, b, c, d) + X(a, b + 1, c, d) + X(a + 1, b + 1, c, d)) / 4.0;
      fp[2][d] = (X(a, b, c + 1, d) + X(a + 1, b, c + 1, d) + X(a, b + 1, c + 1, d) + X(a + 1, b + 1, c + 1, d)) / 4.0;
      fm[1][d] = (X(a, b, c, d) + X(a + 1, b, c, d) + X(a, b, c + 1, d) + X(a + 1, b, c + 1, d)) / 4.0;
      fp[1][d] = (X(a, b + 1, c, d) + X(a + 1, b + 1, c, d) + X(a, b + 1, c + 1, d) + X(a + 1, b + 1, c + 1, d)) / 4.0;
    }
    const double xxi = fp[0][0] - fm[0][0], xet = fp[1][0] - fm[1][0], xzt = fp[2][0] - fm[2][0];
    const double yxi = fp[0][1] - fm[0][1], yet = fp[1][1] - fm[1][1], yzt = fp[2][1] - fm[2][1];
    const double zxi = fp[0][2] - fm[0][2], zet = fp[1][2] - fm[1][2], zzt = fp[2][2] - fm[2][2];
    const double jac = 1.0 / (xxi * (yet * zzt - yzt * zet) + xet * (yzt * zxi - yxi * zzt) +
                              xzt * (yxi * zet - yet * zxi));
    MT(i, j, k, 0, 0) = jac * (yet * zzt - yzt * zet);
    MT(i, j, k, 0, 1) = jac * (xzt * zet - xet * zzt);
    MT(i, j, k, 0, 2) = jac * (xet * yzt - xzt * yet);
    MT(i, j, k, 1, 0) = jac * (yzt * zxi - yxi * zzt);
    MT(i, j, k, 1, 1) = jac * (xxi * zzt - xzt * zxi);
    MT(i, j, k, 1, 2) = jac * (xzt * yxi - xxi * yzt);
    MT(i, j, k, 2, 0) = jac * (yxi * zet - yet * zxi);
    MT(i, j, k, 2, 1) = jac * (xet * zxi - xxi * zet);
    MT(i, j, k, 2, 2) = jac * (xxi * yet - xet * yxi);
  }
  // computeMetrics2D::operator() (src/metric.hpp:30-53)
  void metrics2D(int i, int j) {
    const int a = i - 3, b = j - 3;
    double x_xi = (X(a + 1, b, 0, 0) + X(a + 1, b + 1, 0, 0)) / 2.0 - (X(a, b, 0, 0) + X(a, b + 1, 0, 0)) / 2.0;
    double y_xi = (X(a + 1, b, 0, 1) + X(a + 1, b + 1, 0, 1)) / 2.0 - (X(a, b, 0, 1) + X(a, b + 1, 0, 1)) / 2.0;
    double x_et = (X(a, b + 1, 0, 0) + X(a + 1, b + 1, 0, 0)) / 2.0 - (X(a, b, 0, 0) + X(a + 1, b, 0, 0)) / 2.0;
    double y_et = (X(a, b + 1, 0, 1) + X(a + 1, b + 1, 0, 1)) / 2.0 - (X(a, b, 0, 1) + X(a + 1, b, 0, 1)) / 2.0;
    double jac = 1.0 / (x_xi * y_et - x_et * y_xi);
    MT(i, j, 0, 0, 0) = jac * y_et;
    MT(i, j, 0, 0, 1) = -jac * x_et;
    MT(i, j, 0, 1, 0) = -jac * y_xi;
    MT(i, j, 0, 1, 1) = jac * x_xi;
  }
  // gen3d_func::preSim / gen2d_func::preSim metric setup: interior from the
  // nodes, then the single-rank ghost mirrors (src/gen3d.cpp:278-331 in the
  // order x-, x+, y-, y+, z-, z+; src/gen2d.cpp:280-317 in the order
  // y-, y+, x-, x+), each over the full extent of the other axes.
  void set_grid(const double* X_, size_t n) {
    nodes.assign(X_, X_ + n);
    std::fill(met.begin(), met.end(), 0.0);
    if (ndim == 3)
      box(ng, ngi - ng, ng, ngj - ng, ng, ngk - ng, [&](int i, int j, int k) { metrics3D(i, j, k); });
    else
      box(ng, ngi - ng, ng, ngj - ng, 0, 1, [&](int i, int j, int) { metrics2D(i, j); });
    const int nm = ndim;
    auto copy = [&](int di, int dj, int dk, int si, int sj, int sk) {
      for (int a = 0; a < nm; ++a)
        for (int b = 0; b < nm; ++b) MT(di, dj, dk, a, b) = MT(si, sj, sk, a, b);
    };
    auto mirror_x = [&](int side) {
      for (int g = 0; g < ng; ++g)
        for (int j = 0; j < ngj; ++j)
          for (int k = 0; k < ngk; ++k) {
            if (side == 0) copy(ng - g - 1, j, k, ng + g, j, k);
            else copy(ngi - 1 - g, j, k, nci + g, j, k);
          }
    };
    auto mirror_y = [&](int side) {
      for (int i = 0; i < ngi; ++i)
        for (int g = 0; g < ng; ++g)
          for (int k = 0; k < ngk; ++k) {
            if (side == 0) copy(i, ng - g - 1, k, i, ng + g, k);
            else copy(i, ngj - 1 - g, k, i, ncj + g, k);
          }
    };
    auto mirror_z = [&](int side) {
      for (int i = 0; i < ngi; ++i)
        for (int j = 0; j < ngj; ++j)
          for (int g = 0; g < ng; ++g) {
            if (side == 0) copy(i, j, ng - g - 1, i, j, ng + g);
            else copy(i, j, ngk - 1 - g, i, j, nck + g);
          }
    };
    if (ndim == 3) {
      mirror_x(0); mirror_x(1); mirror_y(0); mirror_y(1); mirror_z(0); mirror_z(1);
    } else {
      mirror_y(0); mirror_y(1); mirror_x(0); mirror_x(1);
    }
  }
  // computeGenVelocity3D (src/velocity.hpp:23-48)
  void genVelocity3D(int i, int j, int k) {
    for (int a = 0; a < 3; ++a)
      VEL(i, j, k, a) = (MT(i, j, k, a, 0) * V(i, j, k, 0) / RHO(i, j, k) +
                         MT(i, j, k, a, 1) * V(i, j, k, 1) / RHO(i, j, k) +
                         MT(i, j, k, a, 2) * V(i, j, k, 2) / RHO(i, j, k));
  }
  // computeGenVelocity2D (src/velocity.hpp:49-66)
  void genVelocity2D(int i, int j) {
    for (int a = 0; a < 2; ++a)
      VEL(i, j, 0, a) = (MT(i, j, 0, a, 0) * V(i, j, 0, 0) / RHO(i, j, 0) +
                         MT(i, j, 0, a, 1) * V(i, j, 0, 1) / RHO(i, j, 0));
  }
  // applyGenPressureGradient3D (src/presgrad.hpp:84-145)
  void genPresgrad3D(int i, int j, int k) {
    for (int w = 0; w < 3; ++w) {
      double dxi = (P(i - 2, j, k) * MT(i - 2, j, k, 0, w) - 8.0 * P(i - 1, j, k) * MT(i - 1, j, k, 0, w) +
                    8.0 * P(i + 1, j, k) * MT(i + 1, j, k, 0, w) - P(i + 2, j, k) * MT(i + 2, j, k, 0, w)) / (12.0);
      double det = (P(i, j - 2, k) * MT(i, j - 2, k, 1, w) - 8.0 * P(i, j - 1, k) * MT(i, j - 1, k, 1, w) +
                    8.0 * P(i, j + 1, k) * MT(i, j + 1, k, 1, w) - P(i, j + 2, k) * MT(i, j + 2, k, 1, w)) / (12.0);
      double dzt = (P(i, j, k - 2) * MT(i, j, k - 2, 2, w) - 8.0 * P(i, j, k - 1) * MT(i, j, k - 1, 2, w) +
                    8.0 * P(i, j, k + 1) * MT(i, j, k + 1, 2, w) - P(i, j, k + 2) * MT(i, j, k + 2, 2, w)) / (12.0);
      D(i, j, k, w) = (D(i, j, k, w) - (dxi + det + dzt));
    }
  }
  // applyGenPressureGradient2D (src/presgrad.hpp:160-189)
  void genPresgrad2D(int i, int j) {
    for (int w = 0; w < 2; ++w) {
      double dxi = (P(i - 2, j, 0) * MT(i - 2, j, 0, 0, w) - 8.0 * P(i - 1, j, 0) * MT(i - 1, j, 0, 0, w) +
                    8.0 * P(i + 1, j, 0) * MT(i + 1, j, 0, 0, w) - P(i + 2, j, 0) * MT(i + 2, j, 0, 0, w)) / (12.0);
      double det = (P(i, j - 2, 0) * MT(i, j - 2, 0, 1, w) - 8.0 * P(i, j - 1, 0) * MT(i, j - 1, 0, 1, w) +
                    8.0 * P(i, j + 1, 0) * MT(i, j + 1, 0, 1, w) - P(i, j + 2, 0) * MT(i, j + 2, 0, 1, w)) / (12.0);
      D(i, j, 0, w) = (D(i, j, 0, w) - (dxi + det));
    }
  }
  // gen3d_func::compute (src/gen3d.cpp:338-370): no BCs
  void computeGen3D() {
    const int b = ng, ei = ngi - ng, ej = ngj - ng, ek = ngk - ng;
    box(0, ngi, 0, ngj, 0, ngk, [&](int i, int j, int k) { rhoPT3D(i, j, k); });
    box(0, ngi, 0, ngj, 0, ngk, [&](int i, int j, int k) { genVelocity3D(i, j, k); });
    for (int v = 0; v < nv; ++v) {
      box(b - 1, ei, b - 1, ej, b - 1, ek, [&](int i, int j, int k) { fluxes3D(i, j, k, v); });
      box(b, ei, b, ej, b, ek, [&](int i, int j, int k) { advect3D(i, j, k, v); });
    }
    box(b, ei, b, ej, b, ek, [&](int i, int j, int k) { genPresgrad3D(i, j, k); });
  }
  // gen2d_func::compute (src/gen2d.cpp:103-130)
  void computeGen2D() {
    const int b = ng, ei = ngi - ng, ej = ngj - ng;
    box(0, ngi, 0, ngj, 0, 1, [&](int i, int j, int) { rhoPT2D(i, j); });
    box(0, ngi, 0, ngj, 0, 1, [&](int i, int j, int) { genVelocity2D(i, j); });
    for (int v = 0; v < nv; ++v) {
      box(b - 1, ei, b - 1, ej, 0, 1, [&](int i, int j, int) { flux2D_any(i, j, v); });
      box(b, ei, b, ej, 0, 1, [&](int i, int j, int) { advect2D(i, j, v); });
    }
    box(b, ei, b, ej, 0, 1, [&](int i, int j, int) { genPresgrad2D(i, j); });
  }
  void get_metrics(double* out) {
    const size_t nc = (size_t)ngi * ngj * ngk;
    for (int b = 0; b < ndim; ++b)
      for (int a = 0; a < ndim; ++a)
        for (int k = 0; k < ngk; ++k)
          for (int j = 0; j < ngj; ++j)
            for (int i = 0; i < ngi; ++i)
              out[(size_t)i + (size_t)ngi * (j + (size_t)ngj * k) + nc * (a + (size_t)ndim * b)] =
                  MT(i, j, k, a, b);
  }

  void compute() {
    if (gen) {
      if (ndim == 3) computeGen3D();
      else computeGen2D();
      return;
    }
    if (ndim == 3) compute3D();
    else compute2D();
  }

  // rkAdvance (src/rk.cpp:28-70), preceded by preStep.
  void rk_step() {
    if (ndim == 2 && !gen) apply_bcs();  // cart2d_func::preStep (src/cart2d.cpp:147-149)
    compute();
    const size_t n = var.size();
    const double hdt = 0.5f * dt;
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < n; ++q) {
      tmp1[q] = var[q];
      var[q] = var[q] + hdt * dvar[q];
    }
    compute();
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < n; ++q) var[q] = tmp1[q] + dt * dvar[q];
  }

  // secondary variables of the current state (postStep path)
  // ---- noise filter: postStep (src/cart3d.cpp:319-374, src/cart2d.cpp:257-307)
  // with detectNoise3D/removeNoise3D and the 2D pair (src/noise.hpp:26-262).
  // Serial, in the MDRange loop order (first index slowest): the removal
  // updates var in place while neighbours read it.
  std::vector<int> noise;  // FS3D_I / FS2D_I, zero-initialised, kept between calls
  inline int& NZ(int i, int j, int k) { return noise[c3(i, j, k)]; }

  void noise_filter(double n_dh, double n_eta, double n_coff, int n_nt, int n_mode) {
    if (noise.empty()) noise.assign((size_t)ngi * ngj * ngk, 0);
    // lattice points per axis: M + 1 in cart3d / cart2d (src/cart3d.cpp:326-339,
    // src/cart2d.cpp:262-272); gen2d_func::postStep (src/gen2d.cpp:150-179)
    // counts from nci - 1, visits M points, uses no cutoff and always
    // filters both momenta
    const bool g2 = gen && ndim == 2;
    const int M = g2 ? ((nci - 1) % 2 == 0 ? (nci - 1) / 2 : nci / 2)
                     : ((nci + 1) % 2 == 0 ? (nci + 1) / 2 : nci / 2);
    const int N = g2 ? ((ncj - 1) % 2 == 0 ? (ncj - 1) / 2 : ncj / 2)
                     : ((ncj + 1) % 2 == 0 ? (ncj + 1) / 2 : ncj / 2);
    const int L = (nck + 1) % 2 == 0 ? (nck + 1) / 2 : nck / 2;
    const int Mn = g2 ? M : M + 1, Nn = g2 ? N : N + 1;
    double coff = 0.0;
    if (cf.ceq && !g2) {
      // 3D: maxCvar3D(var, 6), a fixed variable index; 2D: maxCvar2D(var, 1, cd)
      // = |var(nv+1)|.  Serial max from -DBL_MAX with `s > lmax`.
      const int cv = ndim == 3 ? 6 : nv + 1;
      double mx = -DBL_MAX;
      for (int i = ng; i < ngi - ng; ++i)
        for (int j = ng; j < ngj - ng; ++j)
          for (int k = (ndim == 3 ? ng : 0); k < (ndim == 3 ? ngk - ng : 1); ++k) {
            double s = std::fabs(V(i, j, k, cv));
            if (s > mx) mx = s;
          }
      coff = n_coff * mx;
    }
    std::vector<int> vars;
    if (n_mode == 1 || g2) {
      for (int d = 0; d < ndim; ++d) vars.push_back(d);
    } else {
      vars.push_back(ndim);
    }
    for (int v : vars) {
      if (ndim == 3) {
        for (int ii = 0; ii < M + 1; ++ii)
          for (int jj = 0; jj < N + 1; ++jj)
            for (int kk = 0; kk < L + 1; ++kk) detect3(ii, jj, kk, v, n_dh, coff);
        for (int tau = 0; tau < n_nt; ++tau)
          for (int i = ng; i < ngi - ng; ++i)
            for (int j = ng; j < ngj - ng; ++j)
              for (int k = ng; k < ngk - ng; ++k) {
                const double lap = (V(i - 1, j, k, v) - 2 * V(i, j, k, v) + V(i + 1, j, k, v)) / (dx * dx) +
                                   (V(i, j - 1, k, v) - 2 * V(i, j, k, v) + V(i, j + 1, k, v)) / (dy * dy) +
                                   (V(i, j, k - 1, v) - 2 * V(i, j, k, v) + V(i, j, k + 1, v)) / (dz * dz);
                const double dnoise = n_eta * (dx * dx + dy * dy + dz * dz) * NZ(i, j, k) * lap;
                V(i, j, k, v) += dnoise;
              }
      } else {
        for (int ii = 0; ii < Mn; ++ii)
          for (int jj = 0; jj < Nn; ++jj) detect2(ii, jj, v, n_dh, coff);
        for (int tau = 0; tau < n_nt; ++tau)
          for (int i = ng; i < ngi - ng; ++i)
            for (int j = ng; j < ngj - ng; ++j) {
              const double lgrad = (V(i, j, 0, v) - V(i - 1, j, 0, v)) / dx;
              const double rgrad = (V(i + 1, j, 0, v) - V(i, j, 0, v)) / dx;
              const double bgrad = (V(i, j, 0, v) - V(i, j - 1, 0, v)) / dy;
              const double tgrad = (V(i, j + 1, 0, v) - V(i, j, 0, v)) / dy;
              const double dv = n_eta * (dx * dx + dy * dy) * NZ(i, j, 0) *
                                ((rgrad - lgrad) / dx + (tgrad - bgrad) / dy);
              V(i, j, 0, v) += dv;
            }
      }
    }
  }
  // detectNoise3D at lattice point (ii, jj, kk)
  void detect3(int ii, int jj, int kk, int v, double dh, double coff) {
    const int i = 2 * ii + ng, j = 2 * jj + ng, k = 2 * kk + ng;
    const double a = std::sqrt(165.0 * dx * dy * dz) / 15840.0;
    // the 27 weights in the reference's term order: planes k+1, k, k-1;
    // rows j+1, j, j-1; columns i-1, i, i+1
    static const double w[3][3][3] = {{{2, 2, 2}, {2, 8, 2}, {2, 2, 2}},
                                      {{2, 8, 2}, {8, -88, 8}, {2, 8, 2}},
                                      {{2, 2, 2}, {2, 8, 2}, {2, 2, 2}}};
    double sum = 0.0;
    bool first = true;
    for (int pk = 0; pk < 3; ++pk)
      for (int rj = 0; rj < 3; ++rj)
        for (int ci = 0; ci < 3; ++ci) {
          const double t = w[pk][rj][ci] * V(i - 1 + ci, j + 1 - rj, k + 1 - pk, v);
          sum = first ? t : sum + t;
          first = false;
        }
    const double c = -a * sum;
    const double cref = dh * std::sqrt(dx * dy * dz / 12.0);
    for (int a1 = -1; a1 < 2; ++a1)
      for (int b1 = -1; b1 < 2; ++b1)
        for (int c1 = -1; c1 < 2; ++c1) NZ(i + a1, j + b1, k + c1) = 0;
    if (std::fabs(c) >= cref) {
      for (int a1 = -1; a1 < 2; ++a1)
        for (int b1 = -1; b1 < 2; ++b1)
          for (int c1 = -1; c1 < 2; ++c1)
            if (coff == 0.0 || std::fabs(V(i + a1, j + b1, k + c1, nv + 1)) < coff)
              NZ(i + a1, j + b1, k + c1) = 1;
    }
  }
  // detectNoise2D at lattice point (ii, jj): no abs() on the C_hat test
  void detect2(int ii, int jj, int v, double dh, double coff) {
    const int i = 2 * ii + ng, j = 2 * jj + ng;
    const double a = std::sqrt(6.0 * dx * dy);
    const double c = -(a / 192.0) *
                     (V(i - 1, j + 1, 0, v) + 2 * V(i, j + 1, 0, v) + V(i + 1, j + 1, 0, v) +
                      2 * V(i - 1, j, 0, v) - 12 * V(i, j, 0, v) + 2 * V(i + 1, j, 0, v) +
                      V(i - 1, j - 1, 0, v) + 2 * V(i, j - 1, 0, v) + V(i + 1, j - 1, 0, v));
    const double cref = dh * a / 16.0;
    for (int a1 = -1; a1 < 2; ++a1)
      for (int b1 = -1; b1 < 2; ++b1) NZ(i + a1, j + b1, 0) = 0;
    if (std::fabs(c) >= cref) {
      for (int a1 = -1; a1 < 2; ++a1)
        for (int b1 = -1; b1 < 2; ++b1)
          if (coff == 0.0 || V(i + a1, j + b1, 0, nv + 1) < coff) NZ(i + a1, j + b1, 0) = 1;
    }
  }

  void secondary(double* out, size_t n) {
    const size_t nc = (size_t)ngi * ngj * ngk;
    const int nf = ndim == 3 ? 6 : 5;
    if (ndim == 3) {
      box(0, ngi, 0, ngj, 0, ngk, [&](int i, int j, int k) { rhoPT3D(i, j, k); });
      box(0, ngi, 0, ngj, 0, ngk, [&](int i, int j, int k) { velocity3D(i, j, k); });
    } else {
      box(0, ngi, 0, ngj, 0, 1, [&](int i, int j, int) { rhoPT2D(i, j); });
      box(0, ngi, 0, ngj, 0, 1, [&](int i, int j, int) { velocity2D(i, j); });
    }
    (void)n;
    for (int k = 0; k < ngk; ++k)
      for (int j = 0; j < ngj; ++j)
        for (int i = 0; i < ngi; ++i) {
          size_t L = (size_t)i + (size_t)ngi * (j + (size_t)ngj * k);
          size_t c = c3(i, j, k);
          for (int d = 0; d < ndim; ++d) out[L + nc * d] = vel[c * ndim + d];
          out[L + nc * (ndim + 0)] = p[c];
          out[L + nc * (ndim + 1)] = T[c];
          out[L + nc * (ndim + 2)] = rho[c];
          (void)nf;
        }
  }

  // LayoutLeft <-> LayoutRight repack at the ABI edge
  void from_left(const double* U, std::vector<double>& dst) {
    for (int v = 0; v < nvt; ++v)
      for (int k = 0; k < ngk; ++k)
        for (int j = 0; j < ngj; ++j)
          for (int i = 0; i < ngi; ++i)
            dst[c3(i, j, k) * nvt + v] = U[(size_t)i + (size_t)ngi * (j + (size_t)ngj * (k + (size_t)ngk * v))];
  }
  void to_left(const std::vector<double>& src, double* U) {
    for (int v = 0; v < nvt; ++v)
      for (int k = 0; k < ngk; ++k)
        for (int j = 0; j < ngj; ++j)
          for (int i = 0; i < ngi; ++i)
            U[(size_t)i + (size_t)ngi * (j + (size_t)ngj * (k + (size_t)ngk * v))] = src[c3(i, j, k) * nvt + v];
  }
};

}  // namespace

extern "C" {

struct orc_ctx {
  Oracle o;
};

int orc_create(const fst_config* cfg, orc_ctx** out) {
  if (!cfg || !out) return FST_ERR_INVALID;
  if (cfg->ndim != 2 && cfg->ndim != 3) return FST_ERR_INVALID;
  if (cfg->ng != 3 || cfg->ns < 1 || cfg->ns > FST_MAX_SPECIES) return FST_ERR_INVALID;
  if (cfg->nci < 1 || cfg->ncj < 1 || (cfg->ndim == 3 && cfg->nck < 1)) return FST_ERR_INVALID;
  orc_ctx* c = new orc_ctx();
  c->o.init(cfg);
  *out = c;
  return FST_OK;
}
void orc_destroy(orc_ctx* c) { delete c; }
size_t orc_state_size(const orc_ctx* c) { return c->o.var.size(); }
int orc_set_state(orc_ctx* c, const double* U, size_t n) {
  if (n != c->o.var.size()) return FST_ERR_SIZE;
  c->o.from_left(U, c->o.var);
  return FST_OK;
}
int orc_get_state(orc_ctx* c, double* U, size_t n) {
  if (n != c->o.var.size()) return FST_ERR_SIZE;
  c->o.to_left(c->o.var, U);
  return FST_OK;
}
int orc_apply_bcs(orc_ctx* c) {
  c->o.apply_bcs();
  return FST_OK;
}
int orc_compute_rhs(orc_ctx* c, double* R, size_t n) {
  if (R && n != c->o.var.size()) return FST_ERR_SIZE;
  c->o.compute();
  if (R) c->o.to_left(c->o.dvar, R);
  return FST_OK;
}
int orc_rk_step(orc_ctx* c, int nsteps) {
  for (int s = 0; s < nsteps; ++s) c->o.rk_step();
  return FST_OK;
}
int orc_secondary(orc_ctx* c, double* out, size_t n) {
  size_t need = (size_t)c->o.ngi * c->o.ngj * c->o.ngk * (c->o.ndim == 3 ? 6 : 5);
  if (n != need) return FST_ERR_SIZE;
  c->o.secondary(out, n);
  return FST_OK;
}
int orc_last_max(const orc_ctx* c, double* maxS, double* maxCh) {
  *maxS = c->o.last_maxS;
  *maxCh = c->o.last_maxCh;
  return FST_OK;
}
int orc_noise_filter(orc_ctx* c, const fst_noise_params* np) {
  if (!np) return FST_ERR_INVALID;
  if (c->o.gen && c->o.ndim == 3) return FST_ERR_UNSUPPORTED;  // gen3d has no noise filter
  c->o.noise_filter(np->dh, np->eta, np->coff, np->nt, np->mode);
  return FST_OK;
}
int orc_get_noise(orc_ctx* c, int* out, size_t n) {
  Oracle& o = c->o;
  if (n != (size_t)o.ngi * o.ngj * o.ngk) return FST_ERR_SIZE;
  for (int k = 0; k < o.ngk; ++k)
    for (int j = 0; j < o.ngj; ++j)
      for (int i = 0; i < o.ngi; ++i)
        out[(size_t)i + (size_t)o.ngi * (j + (size_t)o.ngj * k)] =
            o.noise.empty() ? 0 : o.noise[o.c3(i, j, k)];
  return FST_OK;
}
int orc_set_grid(orc_ctx* c, const double* nodes, size_t n) {
  Oracle& o = c->o;
  if (!o.gen) return FST_ERR_UNSUPPORTED;
  if (n != (size_t)o.ni * o.nj * o.nk * 3) return FST_ERR_SIZE;
  o.set_grid(nodes, n);
  return FST_OK;
}
int orc_get_metrics(orc_ctx* c, double* out, size_t n) {
  Oracle& o = c->o;
  if (!o.gen) return FST_ERR_UNSUPPORTED;
  if (n != o.met.size()) return FST_ERR_SIZE;
  o.get_metrics(out);
  return FST_OK;
}
int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

}  // extern "C"
