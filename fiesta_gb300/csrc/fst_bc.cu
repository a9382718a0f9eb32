// fst_bc.cu — device-side ghost fill, replacing applyBCs (src/bc.cpp:179-249)
// and, on one GPU, the MPI halo exchange it starts with (src/bc.cpp:184-187).
//
// Order, as the reference's single-process build runs it: periodic
// self-copies x, y, z (bc_xPer / bc_yPer / bc_zPer, src/bc.cpp:133-176; the
// same result as the ordered halo exchange on one rank), then the face fills
// x-, x+, y-, y+, z-, z+ of bc_gen (src/bc.cpp:33-131), each over the full
// transverse extent so that edges and corners inherit earlier fills.  Axes
// are separate launches because later axes read ghosts written by earlier
// ones; the two faces of an axis share a launch when they touch disjoint
// cells.  One thread owns one ghost line and runs the reference's per-line
// loop in the reference's order.
//
// Built with --fmad=false: the hydrostatic energy extrapolation must round
// exactly as the reference does.
#include "fst_bc_dev.cuh"
#include "fst_internal.h"

namespace {

// bc_xPer / bc_yPer / bc_zPer: thread per (transverse a, transverse b, v).
__global__ void k_periodic(Geo g, double* __restrict__ U, int axis) {
  const int na = axis == 0 ? g.ngj : g.ngi;
  const int nb = axis == 2 ? g.ngj : g.ngk;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long tot = (long long)na * nb * g.nvt;
  if (t >= tot) return;
  fstbc::periodic_line(g, U, axis, (int)(t % na), (int)((t / na) % nb),
                       (int)(t / ((long long)na * nb)));
}

// bc_gen::operator() for one face: thread per transverse (a, b).  With
// blockIdx.y = 0/1 one launch fills both faces of an axis: their lines
// touch disjoint cells when the axis has at least ng interior cells (each
// side reads only its own ng interior layers and writes its own ghosts).
__global__ void k_face(Geo g, double* __restrict__ U, int axis, int side, int type, int type_hi) {
  const int na = axis == 0 ? g.ngj : g.ngi;
  const int nb = axis == 2 ? g.ngj : g.ngk;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)na * nb) return;
  const int sd = gridDim.y == 2 ? (int)blockIdx.y : side;
  fstbc::face_line(g, U, axis, sd, sd ? type_hi : type, (int)(t % na), (int)(t / na));
}

inline unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

// Reset n reduction words to v on the stream (in place of a copy from host
// memory, so that the reset is an ordinary stream-ordered kernel).
__global__ void k_fill_keys(unsigned long long* __restrict__ p, int n, unsigned long long v) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) p[t] = v;
}

}  // namespace

void fst_fill_keys(unsigned long long* p, int n, unsigned long long v, cudaStream_t st) {
  if (n > 0) k_fill_keys<<<nblk(n, 64), 64, 0, st>>>(p, n, v);
}

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
  const int ncell[3] = {g.nci, g.ncj, g.nck};
  for (int ax = 0; ax < g.ndim; ++ax) {
    if (per[ax]) continue;
    long long na = ax == 0 ? g.ngj : g.ngi, nb = ax == 2 ? g.ngj : g.ngk;
    if (ncell[ax] >= g.ng) {  // both faces in one launch
      FST_LAUNCH(prof, "bc_face", stream, launches,
                 k_face<<<dim3(nblk(na * nb, B), 2), B, 0, stream>>>(g, U, ax, 0, types[ax][0],
                                                                    types[ax][1]));
      continue;
    }
    for (int side = 0; side < 2; ++side) {  // x- before x+ (their lines overlap)
      FST_LAUNCH(prof, "bc_face", stream, launches,
                 k_face<<<nblk(na * nb, B), B, 0, stream>>>(g, U, ax, side, types[ax][side],
                                                           types[ax][side]));
    }
  }
  return launches;
}
