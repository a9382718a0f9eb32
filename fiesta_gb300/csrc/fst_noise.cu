// fst_noise.cu — the postStep noise filter (src/cart3d.cpp:319-374,
// src/cart2d.cpp:257-307; detectNoise3D / removeNoise3D and the 2D pair,
// src/noise.hpp:26-262), FP64, bit for bit with the reference's serial run.
//
// Detection: the reference visits a lattice of centres (2ii+ng, 2jj+ng,
// 2kk+ng); each zeroes its 3x3(x3) block of the noise indicator, then sets
// the cells it flags.  Blocks overlap on their faces, so the value a cell
// keeps is the one written by the last block (in loop order) that covers
// it: along each axis the largest covering centre.  k_noise_detect computes
// each centre once (for every filtered variable) and writes the cells it
// owns in that sense.
//
// Removal: var(i,j,k,v) += eta*(dx^2+dy^2+dz^2)*noise*laplacian(var), in
// place, in loop order (i slowest): a cell sees its -x, -y, -z neighbours
// already updated and its +x, +y, +z neighbours not yet.  The same holds
// for a sweep by wavefronts i+j+k = const, which k_noise_remove runs tile by
// tile: one launch per diagonal of 8x8x8 (2D: 16x16) tiles, and inside a
// tile one step per cell wavefront on a shared-memory copy with a one-cell
// halo (tiles on one diagonal share no face).  One launch sweeps every
// filtered variable (each sweep reads and writes its own variable only), and
// a tile without a flagged cell whose values make the update a provable
// no-op skips the wavefront (the FP64 steps are the cost on this part).
//
// Built with --fmad=false; expressions keep the reference's operation order.
#include <cmath>
#include <cstring>

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

// the filtered variables and the detection constants, computed on the host
// with the reference's expressions (products and quotients only, so IEEE
// rounding makes them the same there as on the device)
struct NoiseArgs {
  int nvars, vars[3], M, N, L, nvp1;
  double scale;   // 3D: sqrt(165 dx dy dz)/15840; 2D: sqrt(6 dx dy)/192
  double cref;    // 3D: dh sqrt(dx dy dz/12);      2D: dh sqrt(6 dx dy)/16
  double n_coff;  // the cutoff factor; the cutoff is n_coff * max|C|
};

// One thread per lattice centre (2ii, 2jj, 2kk): the reference's centre
// value c for every filtered variable, then the indicator of the cells whose
// value the serial loop leaves from this centre -- along each axis offsets
// -1 and 0, and +1 for the last centre.  Bit q of the indicator flags
// variable vars[q]; detection of every variable before any removal is the
// reference's order in effect, since removal of one variable touches neither
// another's values nor the C variables the cutoff reads.
template <int NDIM>
__global__ void __launch_bounds__(256) k_noise_detect(Geo g, const double* __restrict__ U,
                                                      int* __restrict__ noise, NoiseArgs A,
                                                      const unsigned long long* __restrict__ key) {
  const int cx = A.M + 1, cy = A.N + 1, cz = NDIM == 3 ? A.L + 1 : 1;
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= (long long)cx * cy * cz) return;
  const int ii = (int)(t % cx), jj = (int)((t / cx) % cy), kk = (int)(t / ((long long)cx * cy));
  const int i = g.ng + 2 * ii, j = g.ng + 2 * jj, k = NDIM == 3 ? g.ng + 2 * kk : 0;
  unsigned hit = 0;
  for (int q = 0; q < A.nvars; ++q) {
    const double* var = U + g.sv * A.vars[q];
    double c;
    if (NDIM == 3) {
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
      c = -A.scale * sum;
    } else {
      auto V = [&](int x, int y) { return var[(long long)x + g.sy * y]; };
      c = -A.scale * (V(i - 1, j + 1) + 2 * V(i, j + 1) + V(i + 1, j + 1) + 2 * V(i - 1, j) -
                      12 * V(i, j) + 2 * V(i + 1, j) + V(i - 1, j - 1) + 2 * V(i, j - 1) +
                      V(i + 1, j - 1));
    }
    if (fabs(c) >= A.cref) hit |= 1u << q;
  }
  const double coff = key ? A.n_coff * fst_unkey(*key) : 0.0;
  const int x1 = ii == A.M, y1 = jj == A.N, z1 = NDIM == 3 && kk == A.L;
  const long long cv = g.sv * (A.nvp1 < g.nvt ? A.nvp1 : 0);  // C_hat (read only if coff != 0)
  for (int dz = NDIM == 3 ? -1 : 0; dz <= z1; ++dz)
    for (int dy = -1; dy <= y1; ++dy)
      for (int dx = -1; dx <= x1; ++dx) {
        const long long cell = (long long)(i + dx) + g.sy * (j + dy) + g.sz * (k + dz);
        int m = (int)hit;
        if (m && coff != 0.0) {
          const double ch = U[cell + cv];
          if (!(NDIM == 3 ? fabs(ch) < coff : ch < coff)) m = 0;  // no abs in 2D
        }
        noise[cell] = m;
      }
}

// the removal's constants; `safe` is the bit pattern of a bound below which
// a tile whose cells are all unflagged is provably left bit for bit as it is
// (0: never skip)
struct RemoveArgs {
  int nvars, vars[3];
  double eta, dx, dy, dz;
  long long safe;
};

// A tile may skip the in-place update of variable q when none of its cells
// is flagged for q and every value it loaded is finite, below `safe` in
// magnitude and not -0: then each laplacian is finite, eta*D*0*lap is a
// signed zero, and x + (+-0) == x bit for bit for every x but -0.
__device__ __forceinline__ bool unsafe_value(double x, long long safe) {
  const long long b = __double_as_longlong(x);
  return (b & 0x7fffffffffffffffll) >= safe || b == (long long)0x8000000000000000ull;
}

// One diagonal (tx+ty+tz = diag) of 8x8x8 interior tiles, 512 threads each,
// every filtered variable in turn.
__global__ void __launch_bounds__(T3* T3* T3) k_noise_remove3(Geo g, double* __restrict__ U,
                                                              const int* __restrict__ noise,
                                                              RemoveArgs R, int diag, int ntx,
                                                              int nty, int ntz) {
  const int tx = blockIdx.x % ntx, ty = blockIdx.x / ntx, tz = diag - tx - ty;
  if (tz < 0 || tz >= ntz) return;  // uniform over the block
  constexpr int E = T3 + 2;
  __shared__ double s[E][E][E];  // [z][y][x], tile + one-cell halo
  const int lx = threadIdx.x, ly = threadIdx.y, lz = threadIdx.z;
  const int i0 = g.ng + T3 * tx - 1, j0 = g.ng + T3 * ty - 1, k0 = g.ng + T3 * tz - 1;
  const int tid = lx + T3 * (ly + T3 * lz);
  const int i = i0 + 1 + lx, j = j0 + 1 + ly, k = k0 + 1 + lz;
  const bool in = i < g.ngi - g.ng && j < g.ngj - g.ng && k < g.ngk - g.ng;
  const long long cell = (long long)i + g.sy * j + g.sz * k;
  const int nzm = in ? noise[cell] : 0;
  const double D = R.dx * R.dx + R.dy * R.dy + R.dz * R.dz;
  for (int q = 0; q < R.nvars; ++q) {
    double* var = U + g.sv * R.vars[q];
    bool busy = in && ((nzm >> q) & 1);
    __syncthreads();  // the previous variable's tile is stored
    for (int p = tid; p < E * E * E; p += T3 * T3 * T3) {
      const int a = p % E, b = (p / E) % E, c = p / (E * E);
      const int x = i0 + a, y = j0 + b, z = k0 + c;
      if (x < g.ngi && y < g.ngj && z < g.ngk) {
        const double val = var[(long long)x + g.sy * y + g.sz * z];
        s[c][b][a] = val;
        busy = busy || unsafe_value(val, R.safe);
      }
    }
    if (!__syncthreads_or(busy)) continue;
    const double nz = (double)((nzm >> q) & 1);
    for (int w = 0; w < 3 * T3 - 2; ++w) {
      if (in && lx + ly + lz == w) {
        const int a = lx + 1, b = ly + 1, c = lz + 1;
        const double lap = (s[c][b][a - 1] - 2 * s[c][b][a] + s[c][b][a + 1]) / (R.dx * R.dx) +
                           (s[c][b - 1][a] - 2 * s[c][b][a] + s[c][b + 1][a]) / (R.dy * R.dy) +
                           (s[c - 1][b][a] - 2 * s[c][b][a] + s[c + 1][b][a]) / (R.dz * R.dz);
        const double dnoise = R.eta * D * nz * lap;
        s[c][b][a] += dnoise;
      }
      __syncthreads();
    }
    if (in) var[cell] = s[lz + 1][ly + 1][lx + 1];
  }
}

// One diagonal (tx+ty = diag) of 16x16 interior tiles, 256 threads each,
// every filtered variable in turn.
__global__ void __launch_bounds__(T2* T2) k_noise_remove2(Geo g, double* __restrict__ U,
                                                          const int* __restrict__ noise,
                                                          RemoveArgs R, int diag, int nty) {
  const int tx = blockIdx.x, ty = diag - tx;
  if (ty < 0 || ty >= nty) return;
  constexpr int E = T2 + 2;
  __shared__ double s[E][E];  // [y][x]
  const int lx = threadIdx.x, ly = threadIdx.y;
  const int i0 = g.ng + T2 * tx - 1, j0 = g.ng + T2 * ty - 1;
  const int tid = lx + T2 * ly;
  const int i = i0 + 1 + lx, j = j0 + 1 + ly;
  const bool in = i < g.ngi - g.ng && j < g.ngj - g.ng;
  const long long cell = (long long)i + g.sy * j;
  const int nzm = in ? noise[cell] : 0;
  const double dx = R.dx, dy = R.dy;
  const double D = dx * dx + dy * dy;
  for (int q = 0; q < R.nvars; ++q) {
    double* var = U + g.sv * R.vars[q];
    bool busy = in && ((nzm >> q) & 1);
    __syncthreads();
    for (int p = tid; p < E * E; p += T2 * T2) {
      const int a = p % E, b = p / E;
      const int x = i0 + a, y = j0 + b;
      if (x < g.ngi && y < g.ngj) {
        const double val = var[(long long)x + g.sy * y];
        s[b][a] = val;
        busy = busy || unsafe_value(val, R.safe);
      }
    }
    if (!__syncthreads_or(busy)) continue;
    const double nz = (double)((nzm >> q) & 1);
    for (int w = 0; w < 2 * T2 - 1; ++w) {
      if (in && lx + ly == w) {
        const int a = lx + 1, b = ly + 1;
        const double lgrad = (s[b][a] - s[b][a - 1]) / dx;
        const double rgrad = (s[b][a + 1] - s[b][a]) / dx;
        const double bgrad = (s[b][a] - s[b - 1][a]) / dy;
        const double tgrad = (s[b + 1][a] - s[b][a]) / dy;
        const double dv = R.eta * D * nz * ((rgrad - lgrad) / dx + (tgrad - bgrad) / dy);
        s[b][a] += dv;
      }
      __syncthreads();
    }
    if (in) var[cell] = s[ly + 1][lx + 1];
  }
}

// the skip bound: with every |value| < 1e290 min(1, dmin^2) each difference
// quotient and laplacian above stays finite; large or non-positive spacings
// or a large eta disable the skip
long long skip_bound(double eta, double dx, double dy, double dz) {
  const double dmin = fmin(fabs(dx), fmin(fabs(dy), fabs(dz)));
  const double dmax = fmax(fabs(dx), fmax(fabs(dy), fabs(dz)));
  if (!(dmin > 0.0) || !(dmax < 1e100) || !(fabs(eta) < 1e100)) return 0;
  const double vs = 1e290 * fmin(1.0, dmin * dmin);
  long long b;
  memcpy(&b, &vs, sizeof(b));
  return b;
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
  NoiseArgs A{};
  if (np.mode == 1 || g2)
    for (int d = 0; d < g.ndim; ++d) A.vars[A.nvars++] = d;
  else
    A.vars[A.nvars++] = g.ndim;
  A.M = M;
  A.N = N;
  A.L = L;
  A.nvp1 = g.nv + 1;
  A.n_coff = np.coff;
  const double dx = cf.dx, dy = cf.dy, dz = g.ndim == 3 ? cf.dz : cf.dx;
  if (g.ndim == 3) {  // detectNoise3D (src/noise.hpp:54, 85)
    A.scale = sqrt(165.0 * dx * dy * dz) / 15840.0;
    A.cref = np.dh * sqrt(dx * dy * dz / 12.0);
  } else {  // detectNoise2D: a = sqrt(6 dx dy), c = -(a/192)(...), cref = dh a/16
    const double a = sqrt(6.0 * dx * dy);
    A.scale = a / 192.0;
    A.cref = np.dh * a / 16.0;
  }
  if (M >= 0 && N >= 0) {  // gen2d with nci or ncj <= 2 has no lattice point
    const long long centres = (long long)(M + 1) * (N + 1) * (g.ndim == 3 ? L + 1 : 1);
    if (g.ndim == 3)
      FST_LAUNCH(prof, "noise_detect", st, n,
                 k_noise_detect<3><<<nblk(centres, 256), 256, 0, st>>>(g, U, noise, A, ceq ? key : nullptr));
    else
      FST_LAUNCH(prof, "noise_detect", st, n,
                 k_noise_detect<2><<<nblk(centres, 256), 256, 0, st>>>(g, U, noise, A, ceq ? key : nullptr));
  }
  RemoveArgs R{A.nvars, {A.vars[0], A.vars[1], A.vars[2]}, np.eta, dx, dy, dz,
               skip_bound(np.eta, dx, dy, g.ndim == 3 ? dz : dy)};
  for (int tau = 0; tau < np.nt; ++tau) {
    if (g.ndim == 3) {
      const int ntx = (g.nci + T3 - 1) / T3, nty = (g.ncj + T3 - 1) / T3, ntz = (g.nck + T3 - 1) / T3;
      for (int d = 0; d <= ntx + nty + ntz - 3; ++d)
        FST_LAUNCH(prof, "noise_remove", st, n,
                   k_noise_remove3<<<ntx * nty, dim3(T3, T3, T3), 0, st>>>(g, U, noise, R, d, ntx,
                                                                           nty, ntz));
    } else {
      const int ntx = (g.nci + T2 - 1) / T2, nty = (g.ncj + T2 - 1) / T2;
      for (int d = 0; d <= ntx + nty - 2; ++d)
        FST_LAUNCH(prof, "noise_remove", st, n,
                   k_noise_remove2<<<ntx, dim3(T2, T2), 0, st>>>(g, U, noise, R, d, nty));
    }
  }
  return n;
}
