// fst_noise.cu — the postStep noise filter (src/cart3d.cpp:319-374,
// src/cart2d.cpp:257-307; detectNoise3D / removeNoise3D and the 2D pair,
// src/noise.hpp:26-262), FP64, bit for bit with the reference's serial run.
//
// Detection: the reference visits a lattice of centres (2ii+ng, 2jj+ng,
// 2kk+ng); each zeroes its 3x3(x3) block of the noise indicator, then sets
// the cells it flags.  Blocks overlap on their faces, so the value a cell
// keeps is the one written by the last block (in loop order) that covers
// it: along each axis the largest covering centre.  k_noise_detect gives
// every covered cell that value directly, one thread per cell.
//
// Removal: var(i,j,k,v) += eta*(dx^2+dy^2+dz^2)*noise*laplacian(var), in
// place, in loop order (i slowest): a cell sees its -x, -y, -z neighbours
// already updated and its +x, +y, +z neighbours not yet.  The same holds
// for a sweep by wavefronts i+j+k = const, which k_noise_remove runs tile by
// tile: one launch per diagonal of 8x8x8 (2D: 16x16) tiles, and inside a
// tile one step per cell wavefront on a shared-memory copy with a one-cell
// halo (tiles on one diagonal share no face).
//
// Built with --fmad=false; expressions keep the reference's operation order.
#include "fst_internal.h"

namespace {

constexpr int T3 = 8;   // 3D tile edge (cells)
constexpr int T2 = 16;  // 2D tile edge

// max |var(cv)| over the interior into key (Kokkos Max semantics: strict
// comparison from -DBL_MAX, NaN skipped)
__global__ void __launch_bounds__(256) k_noise_maxabs(Geo g, const double* __restrict__ U, int cv,
                                                      unsigned long long* __restrict__ key) {
  const double* a = U + g.sv * cv;
  const long long ni = g.nci, nj = g.ncj;
  const long long n = ni * nj * (g.ndim == 3 ? g.nck : 1);
  double mx = -1.7976931348623157e308;
  for (long long t = (long long)blockIdx.x * 256 + threadIdx.x; t < n;
       t += (long long)gridDim.x * 256) {
    const long long i = t % ni, j = (t / ni) % nj, k = t / (ni * nj);
    const double s = fabs(a[(i + g.ng) + g.sy * (j + g.ng) + g.sz * (g.ndim == 3 ? k + g.ng : 0)]);
    if (s > mx) mx = s;
  }
  mx = fst_warp_max(mx);
  __shared__ double sm[8];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w)
      if (sm[w] > mx) mx = sm[w];
    atomicMax(key, fst_key(mx));
  }
}

// the largest lattice centre offset (0, 2, .., 2*Mx) whose 3-wide block
// covers cell offset o (o in [-1, 2*Mx+1])
__device__ __forceinline__ int last_centre(int o, int Mx) {
  if ((o & 1) == 0) return o;
  return o + 1 <= 2 * Mx ? o + 1 : o - 1;
}

struct NoiseArgs {
  int v, M, N, L, nvp1;
  double dh, n_coff, dx, dy, dz;
};

template <int NDIM>
__global__ void __launch_bounds__(256) k_noise_detect(Geo g, const double* __restrict__ U,
                                                      int* __restrict__ noise, NoiseArgs A,
                                                      const unsigned long long* __restrict__ key) {
  const int ex = 2 * A.M + 3, ey = 2 * A.N + 3, ez = NDIM == 3 ? 2 * A.L + 3 : 1;
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= (long long)ex * ey * ez) return;
  const int ox = (int)(t % ex) - 1, oy = (int)((t / ex) % ey) - 1, oz = (int)(t / ((long long)ex * ey)) - 1;
  const int x = g.ng + ox, y = g.ng + oy, z = NDIM == 3 ? g.ng + oz : 0;
  const int i = g.ng + last_centre(ox, A.M), j = g.ng + last_centre(oy, A.N);
  const double* var = U + g.sv * A.v;
  const double coff = key ? A.n_coff * fst_unkey(*key) : 0.0;
  const long long cell = (long long)x + g.sy * y + g.sz * z;
  const long long cq = cell + g.sv * (A.nvp1 < g.nvt ? A.nvp1 : 0);  // C_hat (read only if coff != 0)
  bool flag;
  if (NDIM == 3) {
    const int k = g.ng + last_centre(oz, A.L);
    const double a = sqrt(165.0 * A.dx * A.dy * A.dz) / 15840.0;
    // the reference's 27 terms in its order: planes k+1, k, k-1; rows j+1,
    // j, j-1; columns i-1, i, i+1
    double sum = 0.0;
#pragma unroll
    for (int pk = 0; pk < 3; ++pk)
#pragma unroll
      for (int rj = 0; rj < 3; ++rj)
#pragma unroll
        for (int ci = 0; ci < 3; ++ci) {
          const double w = pk == 1 ? (rj == 1 ? (ci == 1 ? -88.0 : 8.0) : (ci == 1 ? 8.0 : 2.0))
                                   : ((rj == 1 && ci == 1) ? 8.0 : 2.0);
          const double tt = w * var[(long long)(i - 1 + ci) + g.sy * (j + 1 - rj) + g.sz * (k + 1 - pk)];
          sum = (pk == 0 && rj == 0 && ci == 0) ? tt : sum + tt;
        }
    const double c = -a * sum;
    const double cref = A.dh * sqrt(A.dx * A.dy * A.dz / 12.0);
    flag = fabs(c) >= cref && (coff == 0.0 || fabs(U[cq]) < coff);
  } else {
    const double a = sqrt(6.0 * A.dx * A.dy);
    auto V = [&](int ii, int jj) { return var[(long long)ii + g.sy * jj]; };
    const double c = -(a / 192.0) * (V(i - 1, j + 1) + 2 * V(i, j + 1) + V(i + 1, j + 1) +
                                     2 * V(i - 1, j) - 12 * V(i, j) + 2 * V(i + 1, j) +
                                     V(i - 1, j - 1) + 2 * V(i, j - 1) + V(i + 1, j - 1));
    const double cref = A.dh * a / 16.0;
    flag = fabs(c) >= cref && (coff == 0.0 || U[cq] < coff);  // no abs in 2D
  }
  noise[cell] = flag ? 1 : 0;
}

// One diagonal (tx+ty+tz = diag) of 8x8x8 interior tiles, 512 threads each.
__global__ void __launch_bounds__(T3* T3* T3) k_noise_remove3(Geo g, double* __restrict__ U,
                                                              const int* __restrict__ noise, int v,
                                                              double eta, double dx, double dy,
                                                              double dz, int diag, int ntx,
                                                              int nty, int ntz) {
  const int tx = blockIdx.x % ntx, ty = blockIdx.x / ntx, tz = diag - tx - ty;
  if (tz < 0 || tz >= ntz) return;  // uniform over the block
  constexpr int E = T3 + 2;
  __shared__ double s[E][E][E];  // [z][y][x], tile + one-cell halo
  const int lx = threadIdx.x, ly = threadIdx.y, lz = threadIdx.z;
  const int i0 = g.ng + T3 * tx - 1, j0 = g.ng + T3 * ty - 1, k0 = g.ng + T3 * tz - 1;
  double* var = U + g.sv * v;
  const int tid = lx + T3 * (ly + T3 * lz);
  for (int q = tid; q < E * E * E; q += T3 * T3 * T3) {
    const int a = q % E, b = (q / E) % E, c = q / (E * E);
    const int i = i0 + a, j = j0 + b, k = k0 + c;
    if (i < g.ngi && j < g.ngj && k < g.ngk) s[c][b][a] = var[(long long)i + g.sy * j + g.sz * k];
  }
  const int i = i0 + 1 + lx, j = j0 + 1 + ly, k = k0 + 1 + lz;
  const bool in = i < g.ngi - g.ng && j < g.ngj - g.ng && k < g.ngk - g.ng;
  const long long cell = (long long)i + g.sy * j + g.sz * k;
  const int nz = in ? noise[cell] : 0;
  const double D = dx * dx + dy * dy + dz * dz;
  __syncthreads();
  for (int w = 0; w < 3 * T3 - 2; ++w) {
    if (in && lx + ly + lz == w) {
      const int a = lx + 1, b = ly + 1, c = lz + 1;
      const double lap = (s[c][b][a - 1] - 2 * s[c][b][a] + s[c][b][a + 1]) / (dx * dx) +
                         (s[c][b - 1][a] - 2 * s[c][b][a] + s[c][b + 1][a]) / (dy * dy) +
                         (s[c - 1][b][a] - 2 * s[c][b][a] + s[c + 1][b][a]) / (dz * dz);
      const double dnoise = eta * D * nz * lap;
      s[c][b][a] += dnoise;
    }
    __syncthreads();
  }
  if (in) var[cell] = s[lz + 1][ly + 1][lx + 1];
}

// One diagonal (tx+ty = diag) of 16x16 interior tiles, 256 threads each.
__global__ void __launch_bounds__(T2* T2) k_noise_remove2(Geo g, double* __restrict__ U,
                                                          const int* __restrict__ noise, int v,
                                                          double eta, double dx, double dy, int diag,
                                                          int ntx, int nty) {
  const int tx = blockIdx.x, ty = diag - tx;
  if (ty < 0 || ty >= nty) return;
  constexpr int E = T2 + 2;
  __shared__ double s[E][E];  // [y][x]
  const int lx = threadIdx.x, ly = threadIdx.y;
  const int i0 = g.ng + T2 * tx - 1, j0 = g.ng + T2 * ty - 1;
  double* var = U + g.sv * v;
  const int tid = lx + T2 * ly;
  for (int q = tid; q < E * E; q += T2 * T2) {
    const int a = q % E, b = q / E;
    const int i = i0 + a, j = j0 + b;
    if (i < g.ngi && j < g.ngj) s[b][a] = var[(long long)i + g.sy * j];
  }
  const int i = i0 + 1 + lx, j = j0 + 1 + ly;
  const bool in = i < g.ngi - g.ng && j < g.ngj - g.ng;
  const long long cell = (long long)i + g.sy * j;
  const int nz = in ? noise[cell] : 0;
  const double D = dx * dx + dy * dy;
  __syncthreads();
  for (int w = 0; w < 2 * T2 - 1; ++w) {
    if (in && lx + ly == w) {
      const int a = lx + 1, b = ly + 1;
      const double lgrad = (s[b][a] - s[b][a - 1]) / dx;
      const double rgrad = (s[b][a + 1] - s[b][a]) / dx;
      const double bgrad = (s[b][a] - s[b - 1][a]) / dy;
      const double tgrad = (s[b + 1][a] - s[b][a]) / dy;
      const double dv = eta * D * nz * ((rgrad - lgrad) / dx + (tgrad - bgrad) / dy);
      s[b][a] += dv;
    }
    __syncthreads();
  }
  if (in) var[cell] = s[ly + 1][lx + 1];
  (void)ntx;
}

inline unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

int fst_noise_launch(const Geo& g, const fst_config& cf, double* U, int* noise,
                     unsigned long long* key, const fst_noise_params& np, cudaStream_t st,
                     Prof* prof) {
  int n = 0;
  // largest lattice index per axis (src/cart3d.cpp:326-339, src/cart2d.cpp:262-272);
  // gen2d_func::postStep (src/gen2d.cpp:150-179) counts from nci - 1, visits
  // one point fewer, uses no cutoff and always filters both momenta
  const bool g2 = cf.grid_type == FST_GRID_GENERALIZED && g.ndim == 2;
  const int M = g2 ? ((g.nci - 1) % 2 == 0 ? (g.nci - 1) / 2 : g.nci / 2) - 1
                   : ((g.nci + 1) % 2 == 0 ? (g.nci + 1) / 2 : g.nci / 2);
  const int N = g2 ? ((g.ncj - 1) % 2 == 0 ? (g.ncj - 1) / 2 : g.ncj / 2) - 1
                   : ((g.ncj + 1) % 2 == 0 ? (g.ncj + 1) / 2 : g.ncj / 2);
  const int L = (g.nck + 1) % 2 == 0 ? (g.nck + 1) / 2 : g.nck / 2;
  const bool ceq = cf.ceq != 0 && !g2;
  if (ceq) {
    const unsigned long long init = FST_KEY_LOWEST;
    cudaMemcpyAsync(key, &init, sizeof(init), cudaMemcpyHostToDevice, st);
    // 3D: maxCvar3D(var, 6), a fixed index (src/cart3d.cpp:346); 2D: C_hat
    const int cv = g.ndim == 3 ? 6 : g.nv + 1;
    FST_LAUNCH(prof, "noise_max", st, n, k_noise_maxabs<<<152, 256, 0, st>>>(g, U, cv, key));
  }
  int vars[3], nvars = 0;
  if (np.mode == 1 || g2)
    for (int d = 0; d < g.ndim; ++d) vars[nvars++] = d;
  else
    vars[nvars++] = g.ndim;
  const double dz = g.ndim == 3 ? cf.dz : cf.dx;
  for (int q = 0; q < nvars; ++q) {
    NoiseArgs A{vars[q], M, N, L, g.nv + 1, np.dh, np.coff, cf.dx, cf.dy, dz};
    const long long cov = (long long)(2 * M + 3) * (2 * N + 3) * (g.ndim == 3 ? 2 * L + 3 : 1);
    if (M < 0 || N < 0) {
      // no lattice point (gen2d with nci or ncj <= 2): no detection
    } else if (g.ndim == 3)
      FST_LAUNCH(prof, "noise_detect", st, n,
                 k_noise_detect<3><<<nblk(cov, 256), 256, 0, st>>>(g, U, noise, A, ceq ? key : nullptr));
    else
      FST_LAUNCH(prof, "noise_detect", st, n,
                 k_noise_detect<2><<<nblk(cov, 256), 256, 0, st>>>(g, U, noise, A, ceq ? key : nullptr));
    for (int tau = 0; tau < np.nt; ++tau) {
      if (g.ndim == 3) {
        const int ntx = (g.nci + T3 - 1) / T3, nty = (g.ncj + T3 - 1) / T3, ntz = (g.nck + T3 - 1) / T3;
        for (int d = 0; d <= ntx + nty + ntz - 3; ++d)
          FST_LAUNCH(prof, "noise_remove", st, n,
                     k_noise_remove3<<<ntx * nty, dim3(T3, T3, T3), 0, st>>>(
                         g, U, noise, vars[q], np.eta, cf.dx, cf.dy, dz, d, ntx, nty, ntz));
      } else {
        const int ntx = (g.nci + T2 - 1) / T2, nty = (g.ncj + T2 - 1) / T2;
        for (int d = 0; d <= ntx + nty - 2; ++d)
          FST_LAUNCH(prof, "noise_remove", st, n,
                     k_noise_remove2<<<ntx, dim3(T2, T2), 0, st>>>(g, U, noise, vars[q], np.eta,
                                                                   cf.dx, cf.dy, d, ntx, nty));
      }
    }
  }
  return n;
}
