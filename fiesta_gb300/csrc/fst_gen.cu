// fst_gen.cu — metric tensor of a generalized (curvilinear) grid, replacing
// computeMetrics3D / computeMetrics2D (src/metric.hpp:22-166) and the metric
// ghost fills of gen3d_func::preSim / gen2d_func::preSim
// (src/gen3d.cpp:129-335, src/gen2d.cpp:190-320).
//
// Input: node coordinates X(ii, jj, kk, d), LayoutLeft (ni, nj, nk, 3),
// ni = nci + 1.  Output: the metric m(i, j, k, a, b) = d(xi_a)/d(x_b) of
// every cell, LayoutLeft (ngi, ngj, ngk, 3, 3) in 3D and (ngi, ngj, 2, 2) in
// 2D, i.e. met[cell + sv*(a + ndim*b)].
//
// Interior cells: the derivative of x_b along computational direction a is
// the difference of the centroids of the cell's two a-faces (each the mean
// of its four nodes in 3D, two in 2D); the metric is the inverse of that
// Jacobian by cofactors.  Sums run in the reference's order — for the a-face
// of a 3D cell, over the two other axes (p < q) in the order (0,0), (1,0),
// (0,1), (1,1) — and the file is built with --fmad=false, so the values are
// the reference's bit for bit.
//
// Ghost cells: three layers mirrored from the interior, one launch per face
// in the reference's order (3D: x-, x+, y-, y+, z-, z+; 2D: y-, y+, x-, x+),
// each over the full transverse extent so edges and corners copy cells an
// earlier launch filled.  Layer n of the low side copies interior layer n
// (ghost ng-1-n <- ng+n); of the high side, ghost ngi-1-n <- nci+n.
#include "fst_internal.h"

namespace {

struct Nodes {
  const double* X;
  long long ni, nj, nk;
  __device__ __forceinline__ double operator()(long long i, long long j, long long k, int d) const {
    return X[i + ni * (j + nj * (k + nk * d))];
  }
};

// computeMetrics3D::operator() (src/metric.hpp:58-164)
__global__ void __launch_bounds__(128) k_metrics3d(Geo g, Nodes X, double* __restrict__ met) {
  const int i = g.ng + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = g.ng + blockIdx.y;
  const int k = g.ng + blockIdx.z;
  if (i >= g.ngi - g.ng) return;
  const long long ii = i - g.ng, jj = j - g.ng, kk = k - g.ng;
  // face centroid component d of the side-s face normal to axis a
  auto face = [&](int a, int s, int d) {
    long long o[3][4];  // node offsets (i, j, k) of the four corners
    const int p = a == 0 ? 1 : 0, q = a == 2 ? 1 : 2;
    const int cp[4] = {0, 1, 0, 1}, cq[4] = {0, 0, 1, 1};
    for (int n = 0; n < 4; ++n) {
      o[a][n] = s;
      o[p][n] = cp[n];
      o[q][n] = cq[n];
    }
    return (X(ii + o[0][0], jj + o[1][0], kk + o[2][0], d) +
            X(ii + o[0][1], jj + o[1][1], kk + o[2][1], d) +
            X(ii + o[0][2], jj + o[1][2], kk + o[2][2], d) +
            X(ii + o[0][3], jj + o[1][3], kk + o[2][3], d)) /
           4.0;
  };
  double D[3][3];  // D[d][a] = d x_d / d xi_a
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int a = 0; a < 3; ++a) D[d][a] = face(a, 1, d) - face(a, 0, d);
  const double xxi = D[0][0], xet = D[0][1], xzt = D[0][2];
  const double yxi = D[1][0], yet = D[1][1], yzt = D[1][2];
  const double zxi = D[2][0], zet = D[2][1], zzt = D[2][2];
  const double jac = 1.0 / (xxi * (yet * zzt - yzt * zet) + xet * (yzt * zxi - yxi * zzt) +
                            xzt * (yxi * zet - yet * zxi));
  const long long c = fst_idx(g, i, j, k), sv = g.sv;
  auto M = [&](int a, int b) -> double& { return met[c + sv * (a + 3 * b)]; };
  M(0, 0) = jac * (yet * zzt - yzt * zet);
  M(0, 1) = jac * (xzt * zet - xet * zzt);
  M(0, 2) = jac * (xet * yzt - xzt * yet);
  M(1, 0) = jac * (yzt * zxi - yxi * zzt);
  M(1, 1) = jac * (xxi * zzt - xzt * zxi);
  M(1, 2) = jac * (xzt * yxi - xxi * yzt);
  M(2, 0) = jac * (yxi * zet - yet * zxi);
  M(2, 1) = jac * (xet * zxi - xxi * zet);
  M(2, 2) = jac * (xxi * yet - xet * yxi);
}

// computeMetrics2D::operator() (src/metric.hpp:30-53)
__global__ void __launch_bounds__(128) k_metrics2d(Geo g, Nodes X, double* __restrict__ met) {
  const int i = g.ng + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = g.ng + blockIdx.y;
  if (i >= g.ngi - g.ng) return;
  const long long ii = i - g.ng, jj = j - g.ng;
  double x_xi = (X(ii + 1, jj, 0, 0) + X(ii + 1, jj + 1, 0, 0)) / 2.0 -
                (X(ii, jj, 0, 0) + X(ii, jj + 1, 0, 0)) / 2.0;
  double y_xi = (X(ii + 1, jj, 0, 1) + X(ii + 1, jj + 1, 0, 1)) / 2.0 -
                (X(ii, jj, 0, 1) + X(ii, jj + 1, 0, 1)) / 2.0;
  double x_et = (X(ii, jj + 1, 0, 0) + X(ii + 1, jj + 1, 0, 0)) / 2.0 -
                (X(ii, jj, 0, 0) + X(ii + 1, jj, 0, 0)) / 2.0;
  double y_et = (X(ii, jj + 1, 0, 1) + X(ii + 1, jj + 1, 0, 1)) / 2.0 -
                (X(ii, jj, 0, 1) + X(ii + 1, jj, 0, 1)) / 2.0;
  const double jac = 1.0 / (x_xi * y_et - x_et * y_xi);
  const long long c = fst_idx(g, i, j, 0), sv = g.sv;
  met[c] = jac * y_et;            // m(0,0)
  met[c + 2 * sv] = -jac * x_et;  // m(0,1)
  met[c + sv] = -jac * y_xi;      // m(1,0)
  met[c + 3 * sv] = jac * x_xi;   // m(1,1)
}

// One face of the ghost mirror: thread per (layer n, transverse t).
__global__ void k_metric_mirror(Geo g, double* __restrict__ met, int axis, int side, int ncomp) {
  const int ng_[3] = {g.ngi, g.ngj, g.ngk};
  const int nc_[3] = {g.nci, g.ncj, g.nck};
  const int ta = axis == 0 ? 1 : 0, tb = axis == 2 ? 1 : 2;
  const long long na = ng_[ta], nb = g.ndim == 3 ? ng_[tb] : 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= na * nb * g.ng) return;
  const int n = (int)(t % g.ng);
  const long long ab = t / g.ng;
  int idx[3] = {0, 0, 0};
  idx[ta] = (int)(ab % na);
  idx[tb] = (int)(ab / na);
  const int dst = side == 0 ? g.ng - 1 - n : ng_[axis] - 1 - n;
  const int src = side == 0 ? g.ng + n : nc_[axis] + n;
  idx[axis] = dst;
  const long long cd = fst_idx(g, idx[0], idx[1], idx[2]);
  idx[axis] = src;
  const long long cs = fst_idx(g, idx[0], idx[1], idx[2]);
  for (int q = 0; q < ncomp; ++q) met[cd + g.sv * q] = met[cs + g.sv * q];
}

inline unsigned cdiv(long long a, int b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

// Metrics of every cell from the node coordinates; returns launches made.
int fst_gen_metrics(const Geo& g, const double* nodes, double* met, cudaStream_t st) {
  Nodes X{nodes, g.nci + 1LL, g.ncj + 1LL, g.ndim == 3 ? g.nck + 1LL : 1LL};
  int n = 0;
  if (g.ndim == 3) {
    k_metrics3d<<<dim3(cdiv(g.nci, 128), g.ncj, g.nck), 128, 0, st>>>(g, X, met);
  } else {
    k_metrics2d<<<dim3(cdiv(g.nci, 128), g.ncj, 1), 128, 0, st>>>(g, X, met);
  }
  ++n;
  const int ncomp = g.ndim == 3 ? 9 : 4;
  const int order3[3] = {0, 1, 2}, order2[2] = {1, 0};
  for (int q = 0; q < g.ndim; ++q) {
    const int axis = g.ndim == 3 ? order3[q] : order2[q];
    const int ta = axis == 0 ? 1 : 0, tb = axis == 2 ? 1 : 2;
    const int ngs[3] = {g.ngi, g.ngj, g.ngk};
    const long long tot = (long long)ngs[ta] * (g.ndim == 3 ? ngs[tb] : 1) * g.ng;
    for (int side = 0; side < 2; ++side) {
      k_metric_mirror<<<cdiv(tot, 128), 128, 0, st>>>(g, met, axis, side, ncomp);
      ++n;
    }
  }
  return n;
}
