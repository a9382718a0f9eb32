// fst_plain3d.cu — plain FP64 right-hand side of cart3d_func::compute
// (src/cart3d.cpp:220-298) and gen3d_func::compute (src/gen3d.cpp:338-370),
// and the rkAdvance stage combine (src/rk.cpp:28-70) for sm_103a.  On
// generalized grids the primitive pass writes the contravariant velocity and
// the cell pass applies the metric pressure gradient; the flux pass is the
// same WENO5 with the reference's dz = cf.dx (src/gen3d.cpp:359).
//
// The reference runs ~41 Kokkos launches per stage with every intermediate in
// HBM.  Here a stage is four kernels:
//   k_prim3d        rho, p, velocity, mass fractions, internal energy, and the
//                   two global maxima of the C-equation (maxS, maxCh) folded
//                   into the same pass (block max + one atomicMax per block)
//   k_flux3d        WENO5 fluxes of all nv variables on the three faces
//                   owned by each face index (each face computed once; the
//                   face velocity computed once per face, not per variable)
//   k_faces3d       the 27 face velocity gradients, shared by the viscous
//                   stress and the C-equation face terms, which are the same
//                   expressions in the reference
//   k_cell3d        flux divergence, pressure gradient, buoyancy, viscous
//                   divergence x/y/z, C-equation source + diffusion, then the
//                   RK stage combine straight into the next state buffer
// On GB300 the FP64 pipe, not HBM, bounds this path, so the design removes
// repeated FP64 work (species constants hoisted, Y_s and e computed once per
// cell, shared gradients) while keeping every operation the reference
// performs on every value it stores, in the same order.  Built with
// --fmad=false so no a*b+c is contracted: results match the reference's FP64
// run bit for bit.
#include "fst_internal.h"

namespace {

// ---------------------------------------------------------------------------
// k_prim3d: calculateRhoPT3D (src/secondary.hpp:109-151), computeVelocity3D
// (src/velocity.hpp:68-83) over all cells; maxWaveSpeed (src/ceq3d.hpp:25-63)
// and maxGradFunctor(var, nv+1) (src/ceq3d.hpp:82-93) over the interior.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_prim3d(Geo g, Phys P, const double* __restrict__ U,
                                                double* __restrict__ rho, double* __restrict__ pr,
                                                double* __restrict__ vel, double* __restrict__ Y,
                                                double* __restrict__ nrg, double* __restrict__ T,
                                                unsigned long long* __restrict__ red,
                                                const double* __restrict__ met) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long sv = g.sv;
  double lS = -1.7976931348623157e308, lC = -1.7976931348623157e308;
  if (c < sv) {
    double r = 0.0;
    for (int s = 0; s < P.ns; ++s) r = r + U[c + sv * (4 + s)];
    double Cp = 0, Cv = 0;
    for (int s = 0; s < P.ns; ++s) {
      double ys = U[c + sv * (4 + s)] / r;
      Cp = Cp + ys * P.cp_s[s];
      Cv = Cv + ys * P.cv_s[s];
      if (Y) Y[c + sv * s] = ys;
    }
    const double gam = Cp / Cv;
    const double m0 = U[c], m1 = U[c + sv], m2 = U[c + 2 * sv], E = U[c + 3 * sv];
    const double p = (gam - 1) * (E - (0.5 / r) * (m0 * m0 + m1 * m1 + m2 * m2));
    const double u = m0 / r, v = m1 / r, w = m2 / r;
    rho[c] = r;
    pr[c] = p;
    if (met) {
      // computeGenVelocity3D (src/velocity.hpp:23-48): contravariant velocity
      // sum_b m(a,b) * var(b) / rho, metric (a,b) at met[c + sv*(a + 3b)]
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const double* M = met + c + sv * a;
        vel[c + sv * a] = M[0] * m0 / r + M[3 * sv] * m1 / r + M[6 * sv] * m2 / r;
      }
    } else {
      vel[c] = u;
      vel[c + sv] = v;
      vel[c + 2 * sv] = w;
    }
    if (T) T[c] = p / ((Cp - Cv) * r);
    // specific internal energy of calculateRhoGrad::nrg (src/ceq3d.hpp:137-141)
    if (nrg) nrg[c] = E / r - 0.5 * r * (u * u + v * v + w * w);
    if (red) {
      int i = (int)(c % g.sy), j = (int)((c / g.sy) % g.ngj), k = (int)(c / g.sz);
      bool in = i >= g.ng && i < g.ngi - g.ng && j >= g.ng && j < g.ngj - g.ng &&
                k >= g.ng && k < g.ngk - g.ng;
      if (in) {
        double a = sqrt(gam * p / r);
        double s = a + sqrt(m0 * m0 + m1 * m1 + m2 * m2) / r;
        if (s > lS) lS = s;
        double ch = fabs(U[c + sv * (P.nv + 1)]);
        if (ch > lC) lC = ch;
      }
    }
  }
  if (red) {
    lS = fst_warp_max(lS);
    lC = fst_warp_max(lC);
    if ((threadIdx.x & 31) == 0) {
      atomicMax(&red[0], fst_key(lS));
      atomicMax(&red[1], fst_key(lC));
    }
  }
}

// calculateFluxesG::weno (src/flux.hpp:241-266), constants as float literals
__device__ __forceinline__ double weno3d(double f1, double f2, double f3, double f4, double f5) {
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

// ---------------------------------------------------------------------------
// k_flux3d: calculateFluxesG::operator() (src/flux.hpp:268-309) for all v<nv
// on the x, y and z faces at (i+1/2, j, k), (i, j+1/2, k), (i, j, k+1/2),
// face index box [ng-1, ngi-ng) in every dimension.
// F layout: F[(dir*nv + v)*sv + cell].
// The stencil value is var + (v==3)*p.  For v != 3 that is var + 0*p: var
// itself when the six pressures are finite (signed zeros aside, which never
// change a nonzero result), and NaN otherwise; the add is only executed in
// the second case, so NaN propagates exactly as in the reference.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_flux3d(Geo g, Phys P, const double* __restrict__ U,
                                                const double* __restrict__ pr,
                                                const double* __restrict__ vel,
                                                double* __restrict__ F) {
  const int i = g.ng - 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = g.ng - 1 + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = g.ng - 1 + blockIdx.z;
  if (i >= g.ngi - g.ng || j >= g.ngj - g.ng || k >= g.ngk - g.ng) return;
  const long long c = fst_idx(g, i, j, k);
  const long long sv = g.sv;
#pragma unroll 1
  for (int dir = 0; dir < 3; ++dir) {
    const long long s = dir == 0 ? 1 : dir == 1 ? g.sy : g.sz;
    const double* vd = vel + sv * dir;
    const double uf = (-vd[c + 2 * s] + 7.0f * vd[c + s] + 7.0f * vd[c] - vd[c - s]) / 12.0f;
    const DivC dd = dir == 0 ? P.ddx : dir == 1 ? P.ddy : P.ddz;
    double* Fd = F + (long long)dir * P.nv * sv;
    const double p1 = pr[c + 3 * s], p2 = pr[c + 2 * s], p3 = pr[c + s], p4 = pr[c],
                 p5 = pr[c - s], p6 = pr[c - 2 * s];
    const bool pfin = fst_finite(p1) && fst_finite(p2) && fst_finite(p3) && fst_finite(p4) &&
                      fst_finite(p5) && fst_finite(p6);
#pragma unroll 1
    for (int v = 0; v < P.nv; ++v) {
      const double* q = U + sv * v;
      double f1 = q[c + 3 * s], f2 = q[c + 2 * s], f3 = q[c + s], f4 = q[c], f5 = q[c - s],
             f6 = q[c - 2 * s];
      if (v == 3) {
        f1 = f1 + p1; f2 = f2 + p2; f3 = f3 + p3; f4 = f4 + p4; f5 = f5 + p5; f6 = f6 + p6;
      } else if (!pfin) {
        f1 = f1 + 0.0 * p1; f2 = f2 + 0.0 * p2; f3 = f3 + 0.0 * p3;
        f4 = f4 + 0.0 * p4; f5 = f5 + 0.0 * p5; f6 = f6 + 0.0 * p6;
      }
      double wv = uf < 0.0 ? weno3d(f1, f2, f3, f4, f5) : weno3d(f6, f5, f4, f3, f2);
      Fd[sv * v + c] = dd(uf * wv);
    }
  }
}

// ---------------------------------------------------------------------------
// k_faces3d: per face index, the 27 face velocity gradients G[f][d][w]
// (derivative along d of velocity w on face f), then
//  - viscous stress on x/y/z faces: calculateStressTensor{x,y,z}3dv
//    (src/viscosity.hpp:416-459, 499-541, 581-624), S[(f*6+comp)*sv + cell]
//  - C-equation face terms: calculateCeqFaces * calculateCeqGrads
//    (src/ceq3d.hpp:226-332), MF[((f*3+d)*3+w)*sv + cell]
// The reference evaluates each gradient twice (stress and C-equation) with
// the same operations up to operand order of a commutative add, so the
// values are identical and are computed once here.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_faces3d(Geo g, Phys P, const double* __restrict__ U,
                                                 const double* __restrict__ rho,
                                                 const double* __restrict__ vel,
                                                 const double* __restrict__ Y,
                                                 const unsigned long long* __restrict__ red,
                                                 double* __restrict__ S, double* __restrict__ MF) {
  const int i = g.ng - 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = g.ng - 1 + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = g.ng - 1 + blockIdx.z;
  if (i >= g.ngi - g.ng || j >= g.ngj - g.ng || k >= g.ngk - g.ng) return;
  const long long c = fst_idx(g, i, j, k);
  const long long sv = g.sv, sx = 1, sy = g.sy, sz = g.sz;
  double alpha = 0.0;
  if (P.ceq) {
    const double maxCh = fst_unkey(red[1]);
    alpha = (P.dxmag2 / (maxCh + 1.0e-6)) * P.alpha;  // src/cart3d.cpp:285
  }
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    const long long sf = f == 0 ? sx : f == 1 ? sy : sz;  // outward normal step
    double G[3][3];  // G[d][w]
#pragma unroll
    for (int w = 0; w < 3; ++w) {
      const double* u = vel + sv * w;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if (d == f) {
          const DivC dd = d == 0 ? P.ddx : d == 1 ? P.ddy : P.ddz;
          G[d][w] = dd(u[c + sf] - u[c]);
        } else {
          const long long st = d == 0 ? sx : d == 1 ? sy : sz;
          const DivC dd = d == 0 ? P.d4x : d == 1 ? P.d4y : P.d4z;
          G[d][w] = dd((u[c + sf + st] + u[c + st]) - (u[c + sf - st] + u[c - st]));
        }
      }
    }
    if (P.visc) {
      double mu = 0.0;
      for (int s = 0; s < P.ns; ++s)
        mu += ((Y[c + sf + sv * s] + Y[c + sv * s]) / 2.0) * P.mu_s[s];
      const double dudx = G[0][0], dvdx = G[0][1], dwdx = G[0][2];
      const double dudy = G[1][0], dvdy = G[1][1], dwdy = G[1][2];
      const double dudz = G[2][0], dvdz = G[2][1], dwdz = G[2][2];
      double* Sf = S + (long long)f * 6 * sv + c;
      Sf[0 * sv] = (2.0 / 3.0) * mu * (2.0 * dudx - dvdy - dwdz);
      Sf[1 * sv] = (2.0 / 3.0) * mu * (2.0 * dvdy - dudx - dwdz);
      Sf[2 * sv] = (2.0 / 3.0) * mu * (2.0 * dwdz - dudx - dvdy);
      Sf[3 * sv] = mu * (dudy + dvdx);
      Sf[4 * sv] = mu * (dudz + dwdx);
      Sf[5 * sv] = mu * (dvdz + dwdy);
    }
    if (P.ceq) {
      const int nv = P.nv;
      const double r = (rho[c] + rho[c + sf]) / 2.0;
      const double chat = (U[c + sv * (nv + 1)] + U[c + sf + sv * (nv + 1)]) / 2.0;
      double cn[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) cn[q] = (U[c + sv * (nv + 2 + q)] + U[c + sf + sv * (nv + 2 + q)]) / 2.0;
      double cmag = 1.0e-6;
      cmag += cn[0] * cn[0];
      cmag += cn[1] * cn[1];
      cmag += cn[2] * cn[2];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const double dirac = f == d ? 1.0 : 0.0;
        const double M = dirac - (cn[f] * cn[d]) / cmag;
        const double base = alpha * r * chat * M;
        double* MFd = MF + (long long)((f * 3 + d) * 3) * sv + c;
#pragma unroll
        for (int w = 0; w < 3; ++w) MFd[w * sv] = base * G[d][w];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// k_cell3d: per interior cell, the rest of compute() in the reference's
// accumulation order, then the stage combine of rkAdvance:
//   mode 0: R -> Rout (fst_compute_rhs);  mode 1/2: Unew = Uold + coef*R
// advect3D (src/advect.hpp:39-61), applyPressureGradient3D (src/presgrad.hpp:44-71),
// computeBuoyancy3D (src/buoyancy.hpp:22-47), applyViscousTerm{x,y,z}3dv
// (src/viscosity.hpp:460-663), calculateRhoGrad (src/ceq3d.hpp:95-187),
// updateCeq (:189-224), applyCeq (:334-366), Loop1/Loop2 (src/rk.cpp:42-69).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_cell3d(Geo g, Phys P, const double* __restrict__ U,
                                                const double* __restrict__ rho,
                                                const double* __restrict__ pr,
                                                const double* __restrict__ vel,
                                                const double* __restrict__ nrg,
                                                const double* __restrict__ F,
                                                const double* __restrict__ S,
                                                const double* __restrict__ MF,
                                                const unsigned long long* __restrict__ red,
                                                const double* Uold, double* Unew, double coef,
                                                double* __restrict__ Rout,
                                                const double* __restrict__ met) {
  const int i = g.ng + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = g.ng + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = g.ng + blockIdx.z;
  if (i >= g.ngi - g.ng || j >= g.ngj - g.ng || k >= g.ngk - g.ng) return;
  const long long c = fst_idx(g, i, j, k);
  const long long sv = g.sv, sx = 1, sy = g.sy, sz = g.sz;
  const int nv = P.nv;

  auto emit = [&](int v, double R) {
    if (Rout) Rout[c + sv * v] = R;
    else Unew[c + sv * v] = Uold[c + sv * v] + coef * R;
  };
  auto divF = [&](int v) {
    const double* Fx = F + sv * v;
    const double* Fy = F + sv * (nv + v);
    const double* Fz = F + sv * (2 * nv + v);
    return -((Fx[c] - Fx[c - sx]) + (Fy[c] - Fy[c - sy]) + (Fz[c] - Fz[c - sz]));
  };

  double R0 = divF(0), R1 = divF(1), R2 = divF(2), R3 = divF(3);
  // species: only the advective term
  for (int v = 4; v < nv; ++v) emit(v, divF(v));

  if (met) {
    // applyGenPressureGradient3D (src/presgrad.hpp:72-146): fourth-order
    // differences of p * m(a, w) along each computational direction a
    auto d4m = [&](long long st, int a, int w) {
      const double* m = met + sv * (a + 3 * w);
      return (pr[c - 2 * st] * m[c - 2 * st] - 8.0 * pr[c - st] * m[c - st] +
              8.0 * pr[c + st] * m[c + st] - pr[c + 2 * st] * m[c + 2 * st]) /
             12.0;
    };
    R0 = R0 - (d4m(sx, 0, 0) + d4m(sy, 1, 0) + d4m(sz, 2, 0));
    R1 = R1 - (d4m(sx, 0, 1) + d4m(sy, 1, 1) + d4m(sz, 2, 1));
    R2 = R2 - (d4m(sx, 0, 2) + d4m(sy, 1, 2) + d4m(sz, 2, 2));
  } else {  // pressure gradient; the reference uses dz = cd(2) for the z term
    const double dxp = (pr[c - 2 * sx] - 8.0 * pr[c - sx] + 8.0 * pr[c + sx] - pr[c + 2 * sx]) / P.d12x;
    const double dyp = (pr[c - 2 * sy] - 8.0 * pr[c - sy] + 8.0 * pr[c + sy] - pr[c + 2 * sy]) / P.d12y;
    const double dzp = (pr[c - 2 * sz] - 8.0 * pr[c - sz] + 8.0 * pr[c + sz] - pr[c + 2 * sz]) / P.d12pz;
    R0 = R0 - dxp;
    R1 = R1 - dyp;
    R2 = R2 - dzp;
  }
  if (P.buoyancy) {
    const double vb = U[c + sv] / rho[c];
    const double rhop = rho[c] - P.rho_ref;
    const double f = -P.g * rhop;
    R1 += f;
    R3 += vb * f;
  }
  if (P.visc) {
    // stress components feeding (x-mom, y-mom, z-mom) on each face set
    const int comp[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const long long st = f == 0 ? sx : f == 1 ? sy : sz;
      const DivC dd = f == 0 ? P.ddx : f == 1 ? P.ddy : P.ddz;
      const double* Sf = S + (long long)f * 6 * sv;
      const double* u0 = vel;
      const double* u1 = vel + sv;
      const double* u2 = vel + 2 * sv;
      const double ur = (u0[c + st] + u0[c]) / 2.0, ul = (u0[c - st] + u0[c]) / 2.0;
      const double vr = (u1[c + st] + u1[c]) / 2.0, vl = (u1[c - st] + u1[c]) / 2.0;
      const double wr = (u2[c + st] + u2[c]) / 2.0, wl = (u2[c - st] + u2[c]) / 2.0;
      const double s0 = Sf[comp[f][0] * sv + c], s0m = Sf[comp[f][0] * sv + c - st];
      const double s1 = Sf[comp[f][1] * sv + c], s1m = Sf[comp[f][1] * sv + c - st];
      const double s2 = Sf[comp[f][2] * sv + c], s2m = Sf[comp[f][2] * sv + c - st];
      const double a = dd(s0 - s0m);
      const double b = dd(s1 - s1m);
      const double cc = dd(s2 - s2m);
      const double d = dd(ur * s0 - ul * s0m) + dd(vr * s1 - vl * s1m) + dd(wr * s2 - wl * s2m);
      R0 += a;
      R1 += b;
      R2 += cc;
      R3 += d;
    }
  }
  if (P.ceq) {
    // calculateRhoGrad
    auto d4 = [&](const double* a, long long st, double d12) {
      return (a[c - 2 * st] - 8.0 * a[c - st] + 8.0 * a[c + st] - a[c + 2 * st]) / d12;
    };
    const double dxr = d4(rho, sx, P.d12x), dyr = d4(rho, sy, P.d12y), dzr = d4(rho, sz, P.d12z);
    const double dxe = d4(nrg, sx, P.d12x), dye = d4(nrg, sy, P.d12y), dze = d4(nrg, sz, P.d12z);
    const double dxu = d4(vel, sx, P.d12x), dyv = d4(vel + sv, sy, P.d12y),
                 dzw = d4(vel + 2 * sv, sz, P.d12z);
    const double n1 = dxr, n2 = dyr, n3 = dzr;
    const double rgrad = sqrt(dxr * dxr + dyr * dyr + dzr * dzr);
    const double divu = dxu + dyv + dzw;
    const double dnednr = (n1 * dxe + n2 * dye + n3 * dze) * (n1 * dxr + n2 * dyr + n3 * dzr);
    const int ind = dnednr < 0.0 ? 1 : 0;
    double G[5];
    G[0] = divu < 0 ? (1 - ind) * rgrad : 0.0;
    G[1] = ind * rgrad;
    G[2] = dxr;
    G[3] = dyr;
    G[4] = dzr;
    // updateCeq
    const double maxS = fst_unkey(red[0]);
    const double src = maxS / (P.eps * P.dxmag);
    const double dif = P.kap * maxS * P.dxmag;
#pragma unroll
    for (int n = 0; n < 5; ++n) {
      const double* Cn = U + sv * (nv + n);
      const double cc = Cn[c];
      const double lap = P.ddx(Cn[c - sx] - 2 * cc + Cn[c + sx]) +
                         P.ddy(Cn[c - sy] - 2 * cc + Cn[c + sy]) +
                         P.ddz(Cn[c - sz] - 2 * cc + Cn[c + sz]);
      emit(nv + n, src * (G[n] - cc) + dif * lap);
    }
    // applyCeq
    double diffu[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int w = 0; w < 3; ++w) {
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        const long long st = f == 0 ? sx : f == 1 ? sy : sz;
        const DivC dd = f == 0 ? P.ddx : f == 1 ? P.ddy : P.ddz;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const double* m = MF + (long long)((f * 3 + d) * 3 + w) * sv;
          diffu[w] += dd(m[c] - m[c - st]);
        }
      }
    }
    R0 += diffu[0];
    R1 += diffu[1];
    R2 += diffu[2];
  }
  // C-equation variables carried without a right-hand side (the generalized
  // module evolves none): U + coef*0, as the reference's zero dvar gives
  if (!P.ceq)
    for (int v = nv; v < g.nvt; ++v) emit(v, 0.0);
  emit(0, R0);
  emit(1, R1);
  emit(2, R2);
  emit(3, R3);
}

// Stage-1 ghost cells: U1 = U + (0.5*dt)*0 over ghosts (dvar is zero there;
// src/rk.cpp:42-50 runs over every cell).  In 3D the next ghost fill
// rewrites them, except where a periodic copy with fewer interior cells than
// ghost layers reads ghosts; this keeps that case exact too.
__global__ void k_ghost3d(Geo g, const double* __restrict__ Uold, double* __restrict__ Unew,
                          double coef) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.sv) return;
  int i = (int)(c % g.sy), j = (int)((c / g.sy) % g.ngj), k = (int)(c / g.sz);
  bool in = i >= g.ng && i < g.ngi - g.ng && j >= g.ng && j < g.ngj - g.ng && k >= g.ng &&
            k < g.ngk - g.ng;
  if (in) return;
  for (int v = 0; v < g.nvt; ++v) Unew[c + g.sv * v] = Uold[c + g.sv * v] + coef * 0.0;
}

inline unsigned cdiv(long long a, int b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

// One right-hand-side evaluation of Uin (ghosts already filled) followed by
// the chosen output; returns the number of launches.
int fst_plain3d_stage(const Geo& g, const Phys& P, const Plain3DBufs& b, const double* Uin,
                      const double* Uold, double* Unew, double coef, double* Rout, bool ghosts,
                      cudaStream_t st, Prof* prof) {
  int n = 0;
  if (P.ceq) {
    fst_fill_keys(b.red, 2, FST_KEY_LOWEST, st);
  }
  FST_LAUNCH(prof, "prim3d", st, n,
             k_prim3d<<<cdiv(g.sv, 256), 256, 0, st>>>(g, P, Uin, b.rho, b.pr, b.vel,
                                                       P.visc ? b.Y : nullptr,
                                                       P.ceq ? b.nrg : nullptr, nullptr,
                                                       P.ceq ? b.red : nullptr, b.met));
  const dim3 bf(32, 4, 1);
  const dim3 gf(cdiv(g.nci + 1, 32), cdiv(g.ncj + 1, 4), g.nck + 1);
  FST_LAUNCH(prof, "flux3d", st, n, k_flux3d<<<gf, bf, 0, st>>>(g, P, Uin, b.pr, b.vel, b.F));
  if (P.visc || P.ceq) {
    FST_LAUNCH(prof, "faces3d", st, n,
               k_faces3d<<<gf, bf, 0, st>>>(g, P, Uin, b.rho, b.vel, b.Y, b.red, b.S, b.MF));
  }
  const dim3 gc(cdiv(g.nci, 32), cdiv(g.ncj, 4), g.nck);
  FST_LAUNCH(prof, "cell3d", st, n,
             k_cell3d<<<gc, bf, 0, st>>>(g, P, Uin, b.rho, b.pr, b.vel, b.nrg, b.F, b.S, b.MF,
                                         b.red, Uold, Unew, coef, Rout, b.met));
  if (ghosts && !Rout)
    FST_LAUNCH(prof, "ghost3d", st, n,
               k_ghost3d<<<cdiv(g.sv, 256), 256, 0, st>>>(g, Uold, Unew, coef));
  return n;
}

// Secondary variables (postStep path): u, v, w, p, T, rho over all cells.
int fst_plain3d_secondary(const Geo& g, const Phys& P, const Plain3DBufs& b, const double* U,
                          cudaStream_t st) {
  k_prim3d<<<cdiv(g.sv, 256), 256, 0, st>>>(g, P, U, b.rho, b.pr, b.vel, nullptr, nullptr, b.T,
                                            nullptr, nullptr);
  return 1;
}
