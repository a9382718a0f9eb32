// fst_bc_dev.cuh — per-line ghost-fill logic of applyBCs (src/bc.cpp:33-176),
// shared by the single-case launches (fst_bc.cu) and the batched 2D
// ensemble (fst_batch.cu).
#pragma once
#include "fst_common.cuh"

namespace fstbc {

// bc_xPer / bc_yPer / bc_zPer for one (transverse a, transverse b, v) line.
__device__ __forceinline__ void periodic_line(const Geo& g, double* __restrict__ U, int axis,
                                              int a, int b, int v) {
  long long base, st;
  int nc;
  if (axis == 0) {  // a=j, b=k
    base = g.sy * a + g.sz * b + g.sv * v; st = 1; nc = g.nci;
  } else if (axis == 1) {  // a=i, b=k
    base = a + g.sz * b + g.sv * v; st = g.sy; nc = g.ncj;
  } else {  // a=i, b=j
    base = a + g.sy * b + g.sv * v; st = g.sz; nc = g.nck;
  }
  for (int q = 0; q < g.ng; ++q) {
    U[base + st * q] = U[base + st * (nc + q)];
    U[base + st * (nc + g.ng + q)] = U[base + st * (g.ng + q)];
  }
}

// bc_gen::operator() (src/bc.cpp:42-130) for the ghost line through
// transverse (a, b) of one face.
__device__ __forceinline__ void face_line(const Geo& g, double* __restrict__ U, int axis, int side,
                                          int type, int a, int b) {
  const int h = side ? 1 : -1;
  int i, j, k, ih = 0, jh = 0, kh = 0;
  if (axis == 0) { i = side ? g.ng + g.nci - 1 : g.ng; j = a; k = b; ih = h; }
  else if (axis == 1) { i = a; j = side ? g.ng + g.ncj - 1 : g.ng; k = b; jh = h; }
  else { i = a; j = b; k = side ? g.ng + g.nck - 1 : g.ng; kh = h; }
  const long long c0 = fst_idx(g, i, j, k);
  const long long step = ih + g.sy * jh + g.sz * kh;  // one cell outward
  const int ng = g.ng;

  // The copies read only interior cells and write only ghosts, so a chunk of
  // variables is loaded before any of it is stored: the loads are then in
  // flight together (a store through U could alias the next load, which
  // would otherwise serialise them).  Same values as the reference's loop.
  constexpr int CH = 4;  // variables per chunk (with ng = 3: 12 values)
  double x[CH][3];
  for (int v0 = 0; v0 < g.nvt; v0 += CH) {
#pragma unroll
    for (int q = 0; q < CH; ++q)
#pragma unroll
      for (int n = 0; n < 3; ++n)
        if (v0 + q < g.nvt && n < ng) x[q][n] = U[c0 - step * n + g.sv * (v0 + q)];
#pragma unroll
    for (int q = 0; q < CH; ++q) {
      const int v = v0 + q;
      if (v >= g.nvt) break;
      // reflective, hydrostatic (reflect normal momentum) and noslip (all momenta)
      double reflect = 1.0;
      if (type == FST_BC_NOSLIP) {
        if (v == 0 || v == 1 || v == 2) reflect = -1.0;
      } else if (type != FST_BC_OUTFLOW) {
        if (ih != 0 && v == 0) reflect = -1.0;
        if (jh != 0 && v == 1) reflect = -1.0;
        if (kh != 0 && v == 2) reflect = -1.0;
      }
#pragma unroll
      for (int n = 0; n < 3; ++n)
        if (n < ng)
          U[c0 + step * (n + 1) + g.sv * v] =
              type == FST_BC_OUTFLOW ? x[q][n] : reflect * x[q][n];
    }
  }
  for (int n = 3; n < ng; ++n)  // more than 3 ghost layers: the plain loop
    for (int v = 0; v < g.nvt; ++v) {
      double reflect = 1.0;
      if (type == FST_BC_NOSLIP) {
        if (v == 0 || v == 1 || v == 2) reflect = -1.0;
      } else if (type != FST_BC_OUTFLOW) {
        if (ih != 0 && v == 0) reflect = -1.0;
        if (jh != 0 && v == 1) reflect = -1.0;
        if (kh != 0 && v == 2) reflect = -1.0;
      }
      U[c0 + step * (n + 1) + g.sv * v] = reflect * U[c0 - step * n + g.sv * v];
    }
  if (type == FST_BC_OUTFLOW) return;
  if (type != FST_BC_HYDROSTATIC) return;
  // linear extrapolation of internal energy (src/bc.cpp:92-123); density is
  // var(ndim+1), the first species
  const int edx = g.ndim, rdx = g.ndim + 1;
  for (int n = 0; n < ng; ++n) {
    long long cg = c0 + step * (n + 1), c1 = cg - step, c2 = cg - 2 * step;
    double ke = 0, ke1 = 0, ke2 = 0;
    for (int d = 0; d < g.ndim; ++d) {
      double ug = U[cg + g.sv * d], u1 = U[c1 + g.sv * d], u2 = U[c2 + g.sv * d];
      ke += 0.5 * (ug * ug);
      ke1 += 0.5 * (u1 * u1);
      ke2 += 0.5 * (u2 * u2);
    }
    ke = ke / U[cg + g.sv * rdx];
    ke1 = ke1 / U[c1 + g.sv * rdx];
    ke2 = ke2 / U[c2 + g.sv * rdx];
    U[cg + g.sv * edx] = 2 * (U[c1 + g.sv * edx] - ke1) - (U[c2 + g.sv * edx] - ke2) + ke;
  }
}

}  // namespace fstbc
