// fst_bc.cu — device-side ghost fill, replacing applyBCs (src/bc.cpp:179-249)
// and, on one GPU, the MPI halo exchange it starts with (src/bc.cpp:184-187).
//
// Order, as the reference's single-process build runs it: periodic
// self-copies x, y, z (bc_xPer / bc_yPer / bc_zPer, src/bc.cpp:133-176; the
// same result as the ordered halo exchange on one rank), then the face fills
// x-, x+, y-, y+, z-, z+ of bc_gen (src/bc.cpp:33-131), each over the full
// transverse extent so that edges and corners inherit earlier fills.  Every
// step is its own launch because later steps read ghosts written by earlier
// ones.  One thread owns one ghost line and runs the reference's per-line
// loop in the reference's order.
//
// Built with --fmad=false: the hydrostatic energy extrapolation must round
// exactly as the reference does.
#include "fst_internal.h"

namespace {

// bc_xPer / bc_yPer / bc_zPer: thread per (transverse a, transverse b, v).
__global__ void k_periodic(Geo g, double* __restrict__ U, int axis) {
  const int na = axis == 0 ? g.ngj : g.ngi;
  const int nb = axis == 2 ? g.ngj : g.ngk;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long tot = (long long)na * nb * g.nvt;
  if (t >= tot) return;
  int a = (int)(t % na);
  int b = (int)((t / na) % nb);
  int v = (int)(t / ((long long)na * nb));
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

// bc_gen::operator() for one face: thread per transverse (a, b).
__global__ void k_face(Geo g, double* __restrict__ U, int axis, int side, int type) {
  const int na = axis == 0 ? g.ngj : g.ngi;
  const int nb = axis == 2 ? g.ngj : g.ngk;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)na * nb) return;
  int a = (int)(t % na), b = (int)(t / na);
  const int h = side ? 1 : -1;
  int i, j, k, ih = 0, jh = 0, kh = 0;
  if (axis == 0) { i = side ? g.ng + g.nci - 1 : g.ng; j = a; k = b; ih = h; }
  else if (axis == 1) { i = a; j = side ? g.ng + g.ncj - 1 : g.ng; k = b; jh = h; }
  else { i = a; j = b; k = side ? g.ng + g.nck - 1 : g.ng; kh = h; }
  const long long c0 = fst_idx(g, i, j, k);
  const long long step = ih + g.sy * jh + g.sz * kh;  // one cell outward
  const int ng = g.ng;

  if (type == FST_BC_OUTFLOW) {
    for (int v = 0; v < g.nvt; ++v)
      for (int n = 0; n < ng; ++n)
        U[c0 + step * (n + 1) + g.sv * v] = U[c0 - step * n + g.sv * v];
    return;
  }
  // reflective, hydrostatic (reflect normal momentum) and noslip (all momenta)
  for (int v = 0; v < g.nvt; ++v) {
    double reflect = 1.0;
    if (type == FST_BC_NOSLIP) {
      if (v == 0 || v == 1 || v == 2) reflect = -1.0;
    } else {
      if (ih != 0 && v == 0) reflect = -1.0;
      if (jh != 0 && v == 1) reflect = -1.0;
      if (kh != 0 && v == 2) reflect = -1.0;
    }
    for (int n = 0; n < ng; ++n)
      U[c0 + step * (n + 1) + g.sv * v] = reflect * U[c0 - step * n + g.sv * v];
  }
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

inline unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

// Host launcher: the whole applyBCs sequence on `stream`.  Returns the number
// of kernels launched.
int fst_launch_bcs(const Geo& g, const fst_config& cf, double* U, cudaStream_t stream, Prof* prof) {
  int launches = 0;
  const int B = 128;
  const bool per[3] = {cf.xper != 0, cf.yper != 0, g.ndim == 3 && cf.zper != 0};
  for (int ax = 0; ax < g.ndim; ++ax) {
    if (!per[ax]) continue;
    long long na = ax == 0 ? g.ngj : g.ngi, nb = ax == 2 ? g.ngj : g.ngk;
    FST_LAUNCH(prof, "bc_periodic", stream, launches,
               k_periodic<<<nblk(na * nb * g.nvt, B), B, 0, stream>>>(g, U, ax));
  }
  const int types[3][2] = {{cf.bc_xmin, cf.bc_xmax}, {cf.bc_ymin, cf.bc_ymax}, {cf.bc_zmin, cf.bc_zmax}};
  for (int ax = 0; ax < g.ndim; ++ax) {
    if (per[ax]) continue;
    long long na = ax == 0 ? g.ngj : g.ngi, nb = ax == 2 ? g.ngj : g.ngk;
    for (int side = 0; side < 2; ++side) {
      FST_LAUNCH(prof, "bc_face", stream, launches,
                 k_face<<<nblk(na * nb, B), B, 0, stream>>>(g, U, ax, side, types[ax][side]));
    }
  }
  return launches;
}
