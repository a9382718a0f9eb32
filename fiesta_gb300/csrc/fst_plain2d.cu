// fst_plain2d.cu — plain FP64 right-hand side of cart2d_func::compute
// (src/cart2d.cpp:151-237) and gen2d_func::compute (src/gen2d.cpp:103-130),
// and the stage combine of rkAdvance for sm_103a.  The flux pass carries the
// three 2D schemes of both modules (WENO5, centered4, QUICK); on generalized
// grids the primitive pass writes the contravariant velocity and the cell
// pass applies the metric pressure gradient.
//
// Same structure as the 3D path: one pass for primitives and the three
// C-equation maxima, one pass for WENO fluxes, one pass for the viscous and
// C-equation face terms, one pass for the cell update fused with the RK stage.
// The 2D reference differs from 3D in ways kept here on purpose: double
// WENO constants (src/flux.hpp:41-59), constant mu = 2.928e-5 and the
// vel(i,j-1,1) operand in the x-face du/dy (src/viscosity.hpp:62-68), a heat
// flux with k = 0.026 (src/viscosity.hpp:111-136), buoyancy only where
// |rho - rho_ref| >= 1e-6 with |m_y/rho_1| (src/buoyancy.hpp:49-73), the wave
// speed read from a stride-2 species table without /rho (src/ceq.hpp:42-78),
// four C-equation variables with the fifth left unchanged, and no delta term
// in the C-equation face tensor (src/ceq.hpp:200-245).  Built with
// --fmad=false.
#include "fst_internal.h"

namespace {

// calculateRhoPT2D (src/secondary.hpp:60-107), computeVelocity2D
// (src/velocity.hpp:85-99); maxWaveSpeed2D and maxCvar2D(var, 1)
// (src/ceq.hpp:23-78) over the interior.
__global__ void __launch_bounds__(256) k_prim2d(Geo g, Phys P, const double* __restrict__ U,
                                                double* __restrict__ rho, double* __restrict__ pr,
                                                double* __restrict__ vel, double* __restrict__ T,
                                                double* __restrict__ nrg,
                                                unsigned long long* __restrict__ red,
                                                const double* __restrict__ met) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long sv = g.sv;
  double lS = -1.7976931348623157e308, lC = -1.7976931348623157e308;
  if (c < sv) {
    double r = 0.0;
    for (int s = 0; s < P.ns; ++s) r = r + U[c + sv * (3 + s)];
    double Cp = 0, Cv = 0, Cp2 = 0, Cv2 = 0;
    for (int s = 0; s < P.ns; ++s) {
      double ys = U[c + sv * (3 + s)] / r;
      Cp = Cp + ys * P.cp_s[s];
      Cv = Cv + ys * P.cv_s[s];
      if (red) {
        Cp2 = Cp2 + ys * P.cp2_s[s];
        Cv2 = Cv2 + ys * P.cv2_s[s];
      }
    }
    const double gam = Cp / Cv;
    const double m0 = U[c], m1 = U[c + sv], E = U[c + 2 * sv];
    const double p = (gam - 1) * (E - (0.5 / r) * (m0 * m0 + m1 * m1));
    const double u = m0 / r, v = m1 / r;
    rho[c] = r;
    pr[c] = p;
    if (met) {
      // computeGenVelocity2D (src/velocity.hpp:49-66), metric (a,b) at
      // met[c + sv*(a + 2b)]
      vel[c] = met[c] * m0 / r + met[c + 2 * sv] * m1 / r;
      vel[c + sv] = met[c + sv] * m0 / r + met[c + 3 * sv] * m1 / r;
    } else {
      vel[c] = u;
      vel[c + sv] = v;
    }
    if (T) T[c] = p / ((Cp - Cv) * r);
    if (nrg) nrg[c] = E / r - 0.5 * r * (u * u + v * v);
    if (red) {
      int i = (int)(c % g.sy), j = (int)(c / g.sy);
      bool in = i >= g.ng && i < g.ngi - g.ng && j >= g.ng && j < g.ngj - g.ng;
      if (in) {
        const double gam2 = Cp2 / Cv2;
        double a = sqrt(gam2 * p / r);
        double s = a + sqrt(m0 * m0 + m1 * m1);
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

// computeFluxWeno2D::weno (src/flux.hpp:37-63), double constants
__device__ __forceinline__ double weno2d(double f1, double f2, double f3, double f4, double f5) {
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

// computeFluxWeno2D::operator() (src/flux.hpp:65-105) for all v < nv,
// face box [ng-1, ngi-ng) x [ng-1, ngj-ng).  F[(dir*nv + v)*sv + cell].
__global__ void __launch_bounds__(128) k_flux2d(Geo g, Phys P, const double* __restrict__ U,
                                                const double* __restrict__ rho,
                                                const double* __restrict__ pr,
                                                const double* __restrict__ vel,
                                                double* __restrict__ F) {
  const int i = g.ng - 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = g.ng - 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.ngi - g.ng || j >= g.ngj - g.ng) return;
  const long long c = fst_idx(g, i, j, 0);
  const long long sv = g.sv;
  if (P.scheme == FST_SCHEME_CENTERED4) {
    // computeFluxCentered2D (src/flux.hpp:108-167): fourth-order centred
    // face values; face velocity from var(., dir) / rho, p added for the
    // energy only
#pragma unroll 1
    for (int dir = 0; dir < 2; ++dir) {
      const long long s = dir == 0 ? 1 : g.sy;
      const double* m = U + sv * dir;
      const double uf = (0.0 - m[c + 2 * s] / rho[c + 2 * s] + 7.0 * m[c + s] / rho[c + s] +
                         7.0 * m[c] / rho[c] - m[c - s] / rho[c - s]) /
                        12.0;
      const double pf = (0.0 - pr[c + 2 * s] + 7.0 * pr[c + s] + 7.0 * pr[c] - pr[c - s]) / 12.0;
      const DivC dd = dir == 0 ? P.ddx : P.ddy;
      double* Fd = F + (long long)dir * P.nv * sv;
#pragma unroll 1
      for (int v = 0; v < P.nv; ++v) {
        const double* q = U + sv * v;
        double x1 = (0.0 - q[c + 2 * s] + 7.0 * q[c + s] + 7.0 * q[c] - q[c - s]) / 12.0;
        if (v == 2) x1 = x1 + pf;
        Fd[sv * v + c] = dd(uf * x1);
      }
    }
    return;
  }
#pragma unroll 1
  for (int dir = 0; dir < 2; ++dir) {
    const long long s = dir == 0 ? 1 : g.sy;
    const double* vd = vel + sv * dir;
    const double uf = (-vd[c + 2 * s] + 7.0 * vd[c + s] + 7.0 * vd[c] - vd[c - s]) / 12.0;
    const DivC dd = dir == 0 ? P.ddx : P.ddy;
    double* Fd = F + (long long)dir * P.nv * sv;
#pragma unroll 1
    for (int v = 0; v < P.nv; ++v) {
      const double* q = U + sv * v;
      double f1, f2, f3, f4, f5;
      const long long o = uf < 0.0 ? -s : s;  // stencil runs upwind
      const long long c0 = uf < 0.0 ? c + 3 * s : c - 2 * s;
      f1 = q[c0]; f2 = q[c0 + o]; f3 = q[c0 + 2 * o]; f4 = q[c0 + 3 * o]; f5 = q[c0 + 4 * o];
      const double p1 = pr[c0], p2 = pr[c0 + o], p3 = pr[c0 + 2 * o], p4 = pr[c0 + 3 * o],
                   p5 = pr[c0 + 4 * o];
      if (P.scheme == FST_SCHEME_QUICK) {
        // computeFluxQuick2D (src/flux.hpp:169-221): three upwind values
        // f1 = q(c0+o), f2 = q(c0+2o), f3 = q(c0+3o) of the same stencil
        if (v == 2) {
          f2 = f2 + p2; f3 = f3 + p3; f4 = f4 + p4;
        } else if (!(fst_finite(p2) && fst_finite(p3) && fst_finite(p4))) {
          f2 = f2 + 0.0 * p2; f3 = f3 + 0.0 * p3; f4 = f4 + 0.0 * p4;
        }
        Fd[sv * v + c] = dd(uf * (0.75 * f3 + 0.375 * f4 - 0.125 * f2));
        continue;
      }
      if (v == 2) {
        f1 = f1 + p1; f2 = f2 + p2; f3 = f3 + p3; f4 = f4 + p4; f5 = f5 + p5;
      } else if (!(fst_finite(p1) && fst_finite(p2) && fst_finite(p3) && fst_finite(p4) &&
                   fst_finite(p5))) {
        // var + 0*p of the reference: NaN where a pressure is not finite
        f1 = f1 + 0.0 * p1; f2 = f2 + 0.0 * p2; f3 = f3 + 0.0 * p3;
        f4 = f4 + 0.0 * p4; f5 = f5 + 0.0 * p5;
      }
      Fd[sv * v + c] = dd(uf * weno2d(f1, f2, f3, f4, f5));
    }
  }
}

// calculateStressTensor2dv + calculateHeatFlux2dv (src/viscosity.hpp:25-136)
// and computeCeqFlux2D * computeCeqFaces2D (src/ceq.hpp:200-267) on the x and
// y faces of each face index.
// S[(f*3 + {0:xx,1:xy,2:yy})*sv + cell], Q[f*sv + cell],
// MF[((f*2+d)*2+w)*sv + cell].
__global__ void __launch_bounds__(128) k_faces2d(Geo g, Phys P, const double* __restrict__ U,
                                                 const double* __restrict__ rho,
                                                 const double* __restrict__ vel,
                                                 const double* __restrict__ T,
                                                 const unsigned long long* __restrict__ red,
                                                 double* __restrict__ S, double* __restrict__ Q,
                                                 double* __restrict__ MF) {
  const int i = g.ng - 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = g.ng - 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.ngi - g.ng || j >= g.ngj - g.ng) return;
  const long long c = fst_idx(g, i, j, 0);
  const long long sv = g.sv, sx = 1, sy = g.sy;
  const double* u = vel;
  const double* v = vel + sv;
  if (P.visc) {
    const double mu = P.mu2d;
    double dudx, dvdy, dudy, dvdx;
    // x face
    dudx = P.ddx(u[c + sx] - u[c]);
    dvdx = P.ddx(v[c + sx] - v[c]);
    dudy = P.d4y((u[c + sy] + u[c + sx + sy]) - (v[c - sy] + u[c + sx - sy]));
    dvdy = P.d4y((v[c + sy] + v[c + sx + sy]) - (v[c - sy] + v[c + sx - sy]));
    S[0 * sv + c] = (2.0 / 3.0) * mu * (2.0 * dudx - dvdy);
    S[2 * sv + c] = (2.0 / 3.0) * mu * (2.0 * dvdy - dudx);
    S[1 * sv + c] = mu * (dudy + dvdx);
    // y face
    dudx = P.d4x((u[c + sx] + u[c + sx + sy]) - (u[c - sx] + u[c - sx + sy]));
    dvdx = P.d4x((v[c + sx] + v[c + sx + sy]) - (v[c - sx] + v[c - sx + sy]));
    dudy = P.ddy(u[c + sy] - u[c]);
    dvdy = P.ddy(v[c + sy] - v[c]);
    S[3 * sv + c] = (2.0 / 3.0) * mu * (2.0 * dudx - dvdy);
    S[5 * sv + c] = (2.0 / 3.0) * mu * (2.0 * dvdy - dudx);
    S[4 * sv + c] = mu * (dudy + dvdx);
    // heat flux
    Q[c] = P.ddx(-P.kheat2d * (T[c + sx] - T[c]));
    Q[sv + c] = P.ddy(-P.kheat2d * (T[c + sy] - T[c]));
  }
  if (P.ceq) {
    const int nv = P.nv;
    const double maxCh = fst_unkey(red[1]);
    const double alpha = (P.dxmag2 / (maxCh + 1.0e-6)) * P.alpha;  // src/cart2d.cpp:227
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const long long sf = f == 0 ? sx : sy;
      const double r = (rho[c] + rho[c + sf]) / 2.0;
      const double chat = (U[c + sv * (nv + 1)] + U[c + sf + sv * (nv + 1)]) / 2.0;
      double ct[2];
      ct[0] = (U[c + sv * (nv + 2)] + U[c + sf + sv * (nv + 2)]) / 2.0;
      ct[1] = (U[c + sv * (nv + 3)] + U[c + sf + sv * (nv + 3)]) / 2.0;
      const double ctmag = (ct[0] * ct[0] + ct[1] * ct[1]) + 1.0e-6;
#pragma unroll
      for (int w = 0; w < 2; ++w) {
        const double* vw = vel + sv * w;
        double gr[2];
        if (f == 0) {
          gr[0] = P.ddx(vw[c + sx] - vw[c]);
          gr[1] = P.d4y((vw[c + sy] + vw[c + sx + sy]) - (vw[c - sy] + vw[c + sx - sy]));
        } else {
          gr[0] = P.d4x((vw[c + sx] + vw[c + sx + sy]) - (vw[c - sx] + vw[c - sx + sy]));
          gr[1] = P.ddy(vw[c + sy] - vw[c]);
        }
#pragma unroll
        for (int d = 0; d < 2; ++d) {
          const double m = alpha * r * chat * (ct[f] * ct[d]) / ctmag;
          MF[(long long)((f * 2 + d) * 2 + w) * sv + c] = m * gr[d];
        }
      }
    }
  }
}

// Per interior cell: advect2D, applyPressureGradient2D, computeBuoyancy,
// applyViscousTerm2dv, calculateRhoGrad2D, updateCeq2D, applyCeq2D, then the
// stage combine (src/rk.cpp:42-69).
__global__ void __launch_bounds__(128) k_cell2d(Geo g, Phys P, const double* __restrict__ U,
                                                const double* __restrict__ rho,
                                                const double* __restrict__ pr,
                                                const double* __restrict__ vel,
                                                const double* __restrict__ nrg,
                                                const double* __restrict__ F,
                                                const double* __restrict__ S,
                                                const double* __restrict__ Q,
                                                const double* __restrict__ MF,
                                                const unsigned long long* __restrict__ red,
                                                const double* Uold, double* Unew, double coef,
                                                double* __restrict__ Rout,
                                                const double* __restrict__ met) {
  const int i = g.ng + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = g.ng + blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.ngi - g.ng || j >= g.ngj - g.ng) return;
  const long long c = fst_idx(g, i, j, 0);
  const long long sv = g.sv, sx = 1, sy = g.sy;
  const int nv = P.nv;
  auto emit = [&](int v, double R) {
    if (Rout) Rout[c + sv * v] = R;
    else Unew[c + sv * v] = Uold[c + sv * v] + coef * R;
  };
  auto divF = [&](int v) {
    const double* Fx = F + sv * v;
    const double* Fy = F + sv * (nv + v);
    return -((Fx[c] - Fx[c - sx]) + (Fy[c] - Fy[c - sy]));
  };
  double R0 = divF(0), R1 = divF(1), R2 = divF(2);
  for (int v = 3; v < nv; ++v) emit(v, divF(v));
  if (met) {
    // applyGenPressureGradient2D (src/presgrad.hpp:148-190)
    auto d4m = [&](long long st, int a, int w) {
      const double* m = met + sv * (a + 2 * w);
      return (pr[c - 2 * st] * m[c - 2 * st] - 8.0 * pr[c - st] * m[c - st] +
              8.0 * pr[c + st] * m[c + st] - pr[c + 2 * st] * m[c + 2 * st]) /
             12.0;
    };
    R0 = R0 - (d4m(sx, 0, 0) + d4m(sy, 1, 0));
    R1 = R1 - (d4m(sx, 0, 1) + d4m(sy, 1, 1));
  } else {
    const double dxp = (pr[c - 2 * sx] - 8.0 * pr[c - sx] + 8.0 * pr[c + sx] - pr[c + 2 * sx]) / P.d12x;
    const double dyp = (pr[c - 2 * sy] - 8.0 * pr[c - sy] + 8.0 * pr[c + sy] - pr[c + 2 * sy]) / P.d12y;
    R0 -= dxp;
    R1 -= dyp;
  }
  if (P.buoyancy) {
    const double vb = U[c + sv] / U[c + 3 * sv];
    const double rhop = rho[c] - P.rho_ref;
    const double eps = 1e-6;
    if (rhop >= eps || rhop <= -eps) {
      const double f = -P.g * rhop;
      R1 += f;
      R2 += fabs(vb) * f;
    }
  }
  if (P.visc) {
    const double* u = vel;
    const double* v = vel + sv;
    const double ur = (u[c + sx] + u[c]) / 2.0, ul = (u[c - sx] + u[c]) / 2.0;
    const double vr = (v[c + sx] + v[c]) / 2.0, vl = (v[c - sx] + v[c]) / 2.0;
    const double ut = (u[c + sy] + u[c]) / 2.0, ub = (u[c - sy] + u[c]) / 2.0;
    const double vt = (v[c + sy] + v[c]) / 2.0, vb = (v[c - sy] + v[c]) / 2.0;
    const double* sxx = S;
    const double* sxy = S + sv;
    const double* syx = S + 4 * sv;  // stressy(1,0) == stressy(0,1)
    const double* syy = S + 5 * sv;
    const double a = P.ddx(sxx[c] - sxx[c - sx]) + P.ddy(syx[c] - syx[c - sy]);
    const double b = P.ddx(sxy[c] - sxy[c - sx]) + P.ddy(syy[c] - syy[c - sy]);
    const double c1 = P.ddx(ur * sxx[c] - ul * sxx[c - sx]) + P.ddx(vr * sxy[c] - vl * sxy[c - sx]) +
                      P.ddy(ut * syx[c] - ub * syx[c - sy]) + P.ddy(vt * syy[c] - vb * syy[c - sy]);
    const double c2 = P.ddx(Q[c] - Q[c - sx]) + P.ddy(Q[sv + c] - Q[sv + c - sy]);
    R0 = R0 + a;
    R1 = R1 + b;
    R2 = R2 + c1 - c2;
  }
  if (P.ceq) {
    auto d4 = [&](const double* a, long long st, double d12) {
      return (a[c - 2 * st] - 8.0 * a[c - st] + 8.0 * a[c + st] - a[c + 2 * st]) / d12;
    };
    const double dxr = d4(rho, sx, P.d12x), dyr = d4(rho, sy, P.d12y);
    const double dxe = d4(nrg, sx, P.d12x), dye = d4(nrg, sy, P.d12y);
    const double dxu = d4(vel, sx, P.d12x), dyv = d4(vel + sv, sy, P.d12y);
    const double n1 = dxr, n2 = dyr;
    const double rgrad = sqrt(dxr * dxr + dyr * dyr);
    const double divu = dxu + dyv;
    const double dnednr = (n1 * dxe + n2 * dye) * (n1 * dxr + n2 * dyr);
    const double i1 = dnednr < 0.0 ? 1.0 : 0.0;
    const double i2 = divu < 0.0 ? 1.0 : 0.0;
    double G[4];
    G[0] = (1 - i1) * i2 * rgrad;
    G[1] = i1 * rgrad;
    G[2] = -dyr;
    G[3] = dxr;
    const double maxS = fst_unkey(red[0]);
    const double src = maxS / (P.eps * P.dxmag);
    const double dif = P.kap * maxS * P.dxmag;
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      const double* Cn = U + sv * (nv + n);
      const double cc = Cn[c];
      const double dx_right = P.ddx(Cn[c + sx] - cc);
      const double dx_left = P.ddx(cc - Cn[c - sx]);
      const double dy_top = P.ddy(Cn[c + sy] - cc);
      const double dy_bot = P.ddy(cc - Cn[c - sy]);
      const double lap = dx_right - dx_left + dy_top - dy_bot;
      emit(nv + n, src * (G[n] - cc) + dif * lap);
    }
    emit(nv + 4, 0.0);  // the fifth C variable has no right-hand side
#pragma unroll
    for (int w = 0; w < 2; ++w) {
      const double* m00 = MF + (long long)(0 * 2 + w) * sv;
      const double* m01 = MF + (long long)(2 + w) * sv;
      const double* m10 = MF + (long long)(4 + w) * sv;
      const double* m11 = MF + (long long)(6 + w) * sv;
      double diffu = 0;
      diffu += P.ddx(m00[c] - m00[c - sx]);
      diffu += P.ddx(m01[c] - m01[c - sx]);
      diffu += P.ddy(m10[c] - m10[c - sy]);
      diffu += P.ddy(m11[c] - m11[c - sy]);
      if (w == 0) R0 += diffu;
      else R1 += diffu;
    }
  }
  // C-equation variables carried without a right-hand side (the generalized
  // module evolves none): U + coef*0, as the reference's zero dvar gives
  if (!P.ceq)
    for (int v = nv; v < g.nvt; ++v) emit(v, 0.0);
  emit(0, R0);
  emit(1, R1);
  emit(2, R2);
}

// Stage-1 ghost cells: U1 = U + (0.5*dt)*0 over ghosts (dvar is zero there;
// src/rk.cpp:42-50 runs over every cell).  2D BCs are applied once per step,
// so stage 2 reads these.
__global__ void k_ghost2d(Geo g, const double* __restrict__ Uold, double* __restrict__ Unew,
                          double coef) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.sv) return;
  int i = (int)(c % g.sy), j = (int)(c / g.sy);
  bool in = i >= g.ng && i < g.ngi - g.ng && j >= g.ng && j < g.ngj - g.ng;
  if (in) return;
  for (int v = 0; v < g.nvt; ++v) Unew[c + g.sv * v] = Uold[c + g.sv * v] + coef * 0.0;
}

inline unsigned cdiv(long long a, int b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

int fst_plain2d_stage(const Geo& g, const Phys& P, const Plain2DBufs& b, const double* Uin,
                      const double* Uold, double* Unew, double coef, double* Rout, bool ghosts,
                      cudaStream_t st, Prof* prof) {
  int n = 0;
  if (P.ceq) {
    fst_fill_keys(b.red, 2, FST_KEY_LOWEST, st);
  }
  FST_LAUNCH(prof, "prim2d", st, n,
             k_prim2d<<<cdiv(g.sv, 256), 256, 0, st>>>(g, P, Uin, b.rho, b.pr, b.vel,
                                                       P.visc ? b.T : nullptr,
                                                       P.ceq ? b.nrg : nullptr,
                                                       P.ceq ? b.red : nullptr, b.met));
  const dim3 bf(32, 4, 1);
  const dim3 gf(cdiv(g.nci + 1, 32), cdiv(g.ncj + 1, 4), 1);
  FST_LAUNCH(prof, "flux2d", st, n,
             k_flux2d<<<gf, bf, 0, st>>>(g, P, Uin, b.rho, b.pr, b.vel, b.F));
  if (P.visc || P.ceq) {
    FST_LAUNCH(prof, "faces2d", st, n,
               k_faces2d<<<gf, bf, 0, st>>>(g, P, Uin, b.rho, b.vel, b.T, b.red, b.S, b.Q, b.MF));
  }
  const dim3 gc(cdiv(g.nci, 32), cdiv(g.ncj, 4), 1);
  FST_LAUNCH(prof, "cell2d", st, n,
             k_cell2d<<<gc, bf, 0, st>>>(g, P, Uin, b.rho, b.pr, b.vel, b.nrg, b.F, b.S, b.Q,
                                         b.MF, b.red, Uold, Unew, coef, Rout, b.met));
  if (ghosts && !Rout) {
    FST_LAUNCH(prof, "ghost2d", st, n,
               k_ghost2d<<<cdiv(g.sv, 256), 256, 0, st>>>(g, Uold, Unew, coef));
  }
  return n;
}

int fst_plain2d_secondary(const Geo& g, const Phys& P, const Plain2DBufs& b, const double* U,
                          cudaStream_t st) {
  k_prim2d<<<cdiv(g.sv, 256), 256, 0, st>>>(g, P, U, b.rho, b.pr, b.vel, b.T, nullptr, nullptr,
                                            nullptr);
  return 1;
}
