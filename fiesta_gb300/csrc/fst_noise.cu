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
// tile: one launch per diagonal of 8x8x8 (2D: 32x32) tiles, and inside a
// tile one step per cell wavefront on a shared-memory copy with a one-cell
// halo (tiles on one diagonal share no face).  Each tile sweeps every
// filtered variable side by side (each sweep reads and writes its own
// variable only).  A tile without a flagged cell whose values make the
// update a provable no-op skips its wavefronts, and k_noise_tiles marks in
// one launch the tiles that cannot skip, so the others return at once (the
// FP64 steps are the cost on this part).
//
// Built with --fmad=false; expressions keep the reference's operation order.
#include <cmath>
#include <cstring>

#include "fst_internal.h"

namespace {

constexpr int T3 = 8;   // 3D tile edge (cells)
constexpr int T2 = 32;  // 2D tile edge

// max |var(cv)| over the interior into key (Kokkos Max semantics: strict
// comparison from -DBL_MAX, NaN skipped)
__global__ void __launch_bounds__(256) k_noise_maxabs(Geo g, const double* __restrict__ U, int cv,
                                                      unsigned long long* __restrict__ key) {
  const double* a = U + g.sv * cv;
  const int rows = g.ncj * (g.ndim == 3 ? g.nck : 1);
  // per-thread maximum on the integer key of |value| (an FP64 compare would
  // run on the FP64 pipe); NaN skipped
  unsigned long long kmx = FST_KEY_LOWEST;
  constexpr int RB = 4;  // interior rows per step, their loads in flight together
  for (int r0 = blockIdx.x * RB; r0 < rows; r0 += gridDim.x * RB)
    for (int i = threadIdx.x; i < g.nci; i += 256) {
      unsigned long long v[RB];
#pragma unroll
      for (int u = 0; u < RB; ++u) {  // a row past the end repeats the first one
        const int r = r0 + u < rows ? r0 + u : 0, j = r % g.ncj, k = r / g.ncj;
        v[u] = fst_bits(a[g.ng + i + g.sy * (j + g.ng) + g.sz * (g.ndim == 3 ? k + g.ng : 0)]) &
               0x7FFFFFFFFFFFFFFFull;
      }
#pragma unroll
      for (int u = 0; u < RB; ++u)
        if (v[u] <= 0x7FF0000000000000ull) {  // not NaN; |value| keys as value | sign bit
          const unsigned long long key = v[u] | 0x8000000000000000ull;
          kmx = key > kmx ? key : kmx;
        }
    }
  double mx = fst_unkey(kmx);
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

// the filtered variables and the detection constants, computed on the host
// with the reference's expressions (products and quotients only, so IEEE
// rounding makes them the same there as on the device)
// the weight of term n (planes k+1, k, k-1; rows j+1, j, j-1; columns i-1,
// i, i+1) of the 3D detection stencil: -88 at the centre, 8 on the six face
// neighbours, 2 elsewhere
__device__ __forceinline__ double stencil_weight(int n) {
  const int pk = n / 9, rj = (n / 3) % 3, ci = n % 3;
  return pk == 1 ? (rj == 1 ? (ci == 1 ? -88.0 : 8.0) : (ci == 1 ? 8.0 : 2.0))
                 : ((rj == 1 && ci == 1) ? 8.0 : 2.0);
}

// vars[q] without a local-memory copy of the kernel parameter
__device__ __forceinline__ int pick(const int (&v)[3], int q) { return q == 0 ? v[0] : q == 1 ? v[1] : v[2]; }

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
    const double* var = U + g.sv * pick(A.vars, q);
    double c;
    if (NDIM == 3) {
      // the reference's 27 terms in its order: planes k+1, k, k-1; rows j+1,
      // j, j-1; columns i-1, i, i+1
      double t[27];
      unsigned emax = 0;  // largest biased exponent of the 27 values
#pragma unroll
      for (int n = 0; n < 27; ++n) {
        const int pk = n / 9, rj = (n / 3) % 3, ci = n % 3;
        t[n] = var[(long long)(i - 1 + ci) + g.sy * (j + 1 - rj) + g.sz * (k + 1 - pk)];
        emax = max(emax, (unsigned)(fst_bits(t[n]) >> 52) & 0x7ffu);
      }
      double sum = 2.0 * t[0];
      if (emax < 1023 + 1020) {
        // every |value| < 2^1020: the weights 2 and 8 scale exactly, so
        // fma(w, v, sum) rounds sum + w*v once, as the reference's
        // sum + (w*v) does -- the same bits for half the FP64 operations
#pragma unroll
        for (int n = 1; n < 27; ++n)
          sum = n == 13 ? sum + -88.0 * t[n] : __fma_rn(stencil_weight(n), t[n], sum);
      } else {
#pragma unroll
        for (int n = 1; n < 27; ++n) sum = sum + stencil_weight(n) * t[n];
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
  const unsigned long long b = fst_bits(x);
  return (b & 0x7fffffffffffffffull) >= (unsigned long long)safe || b == 0x8000000000000000ull;
}

// OR of `bits` over the block, written by thread 0 to *out
__device__ __forceinline__ void block_or_store(unsigned bits, int* out) {
  __shared__ unsigned acc;
  if (threadIdx.x == 0) acc = 0;
  __syncthreads();
  const unsigned w = __reduce_or_sync(0xffffffffu, bits);
  if ((threadIdx.x & 31) == 0 && w) atomicOr(&acc, w);
  __syncthreads();
  if (threadIdx.x == 0) *out = (int)acc;
}

// The tiles a removal sweep must visit, bit q for variable vars[q]: a cell
// flagged for q, or a value of q in the tile or its one-cell halo that
// unsafe_value does not clear.  Any other tile is left bit for bit by the
// sweep, as long as its halo stays safe: a visited tile that leaves an
// unsafe value marks its face neighbours (k_noise_remove*).  One block per
// tile, every tile in one launch.
__global__ void __launch_bounds__(256) k_noise_tiles3(Geo g, const double* __restrict__ U,
                                                      const int* __restrict__ noise,
                                                      int* __restrict__ tiles, RemoveArgs R,
                                                      int ntx, int nty) {
  constexpr int E = T3 + 2, NL = (E * E * E + 255) / 256;
  const int tx = blockIdx.x % ntx, ty = (blockIdx.x / ntx) % nty, tz = blockIdx.x / (ntx * nty);
  const int i0 = g.ng + T3 * tx - 1, j0 = g.ng + T3 * ty - 1, k0 = g.ng + T3 * tz - 1;
  const int xe = min(T3, g.ngi - g.ng - (i0 + 1)), ye = min(T3, g.ngj - g.ng - (j0 + 1)),
            ze = min(T3, g.ngk - g.ng - (k0 + 1));
  const int tid = threadIdx.x;
  unsigned bits = 0;
  for (int p = tid; p < T3 * T3 * T3; p += 256) {
    const int x = p % T3, y = (p / T3) % T3, z = p / (T3 * T3);
    if (x < xe && y < ye && z < ze)
      bits |= (unsigned)noise[(long long)(i0 + 1 + x) + g.sy * (j0 + 1 + y) + g.sz * (k0 + 1 + z)];
  }
  bits &= (1u << R.nvars) - 1;
  for (int q = 0; q < R.nvars; ++q) {
    const double* var = U + g.sv * pick(R.vars, q);
    bool bad = false;
#pragma unroll
    for (int u = 0; u < NL; ++u) {
      const int p = tid + 256 * u;
      const int x = i0 + p % E, y = j0 + (p / E) % E, z = k0 + p / (E * E);
      if (p < E * E * E && x < g.ngi && y < g.ngj && z < g.ngk)
        bad = bad || unsafe_value(var[(long long)x + g.sy * y + g.sz * z], R.safe);
    }
    if (bad) bits |= 1u << q;
  }
  block_or_store(bits, tiles + blockIdx.x);
}

__global__ void __launch_bounds__(256) k_noise_tiles2(Geo g, const double* __restrict__ U,
                                                      const int* __restrict__ noise,
                                                      int* __restrict__ tiles, RemoveArgs R,
                                                      int ntx) {
  constexpr int E = T2 + 2, NL = (E * E + 255) / 256;
  const int tx = blockIdx.x % ntx, ty = blockIdx.x / ntx;
  const int i0 = g.ng + T2 * tx - 1, j0 = g.ng + T2 * ty - 1;
  const int xe = min(T2, g.ngi - g.ng - (i0 + 1)), ye = min(T2, g.ngj - g.ng - (j0 + 1));
  const int tid = threadIdx.x;
  unsigned bits = 0;
  for (int p = tid; p < T2 * T2; p += 256) {
    const int x = p % T2, y = p / T2;
    if (x < xe && y < ye) bits |= (unsigned)noise[(long long)(i0 + 1 + x) + g.sy * (j0 + 1 + y)];
  }
  bits &= (1u << R.nvars) - 1;
  for (int q = 0; q < R.nvars; ++q) {
    const double* var = U + g.sv * pick(R.vars, q);
    bool bad = false;
#pragma unroll
    for (int u = 0; u < NL; ++u) {
      const int p = tid + 256 * u;
      const int x = i0 + p % E, y = j0 + p / E;
      if (p < E * E && x < g.ngi && y < g.ngj)
        bad = bad || unsafe_value(var[(long long)x + g.sy * y], R.safe);
    }
    if (bad) bits |= 1u << q;
  }
  block_or_store(bits, tiles + blockIdx.x);
}

// after a visited tile's update: if it left a value unsafe for its
// neighbours' skip (non-finite or large; -0 matters to its own cells only),
// mark the face neighbours for variable q -- later diagonals of this sweep
// and, for the earlier ones, the next sweep
__device__ __forceinline__ bool hard_value(double x, long long safe) {
  return (fst_bits(x) & 0x7fffffffffffffffull) >= (unsigned long long)safe;
}

// cells of an 8-cube with x+y+z = s, ordered by z then y: those in plane z
// number c(s - z), c(u) = min(u, 7) - max(0, u - 7) + 1 for 0 <= u <= 14
__device__ __forceinline__ int row_cells(int u) {
  return u < 0 || u > 2 * T3 - 2 ? 0 : min(u, T3 - 1) - max(0, u - (T3 - 1)) + 1;
}

constexpr int R3 = 256;  // threads per 3D tile: up to three variables x 64 threads in a step

// OR of per-thread bits over the block into *acc (zeroed before a barrier)
__device__ __forceinline__ void or_into(unsigned* acc, unsigned bits) {
  const unsigned w = __reduce_or_sync(0xffffffffu, bits);
  if ((threadIdx.x & 31) == 0 && w) atomicOr(acc, w);
}

// One diagonal (tx+ty+tz = diag) of 8x8x8 interior tiles.  The filtered
// variables are swept side by side: threads 64q .. 64q+63 run variable q's
// wavefront steps (each variable's sweep reads and writes only its own
// values), with the cells of wavefront w in consecutive threads (a table in
// shared memory), so a step's FP64 work occupies ceil(cells/32) warps per
// variable rather than every warp the wavefront crosses.
__global__ void __launch_bounds__(R3, 3) k_noise_remove3(Geo g, double* __restrict__ U,
                                                         const int* __restrict__ noise,
                                                         int* __restrict__ tiles, RemoveArgs R,
                                                         int diag, int ntx, int nty, int ntz) {
  const int tx = blockIdx.x % ntx, ty = blockIdx.x / ntx, tz = diag - tx - ty;
  if (tz < 0 || tz >= ntz) return;  // uniform over the block
  const int tile = blockIdx.x + ntx * nty * tz;
  const unsigned cand = (unsigned)tiles[tile];
  if (!cand) return;  // no variable to visit (k_noise_tiles3)
  constexpr int E = T3 + 2, C = T3 * T3 * T3, W = 3 * T3 - 2, E3 = E * E * E;
  __shared__ double s[3][E][E][E];       // per variable: [z][y][x], tile + one-cell halo
  __shared__ int msk[C];                 // indicator of the tile's cells (0 outside)
  __shared__ unsigned short order[C];    // cells (x + 8y + 64z) by wavefront
  __shared__ short off[W + 1];           // wavefront w: order[off[w] .. off[w+1])
  __shared__ unsigned busy_s, hard_s;
  const int tid = threadIdx.x;
  const int i0 = g.ng + T3 * tx - 1, j0 = g.ng + T3 * ty - 1, k0 = g.ng + T3 * tz - 1;
  const int xe = min(T3, g.ngi - g.ng - (i0 + 1)), ye = min(T3, g.ngj - g.ng - (j0 + 1)),
            ze = min(T3, g.ngk - g.ng - (k0 + 1));  // interior extent of the tile
  if (tid == 0) busy_s = hard_s = 0;
  unsigned bits = 0;
  for (int p = tid; p < C; p += R3) {
    const int x = p % T3, y = (p / T3) % T3, z = p / (T3 * T3);
    const int m = x < xe && y < ye && z < ze
                      ? noise[(long long)(i0 + 1 + x) + g.sy * (j0 + 1 + y) + g.sz * (k0 + 1 + z)]
                      : 0;
    msk[p] = m;
    bits |= (unsigned)m;
  }
  for (int q = 0; q < R.nvars; ++q) {
    if (!((cand >> q) & 1)) continue;
    const double* var = U + g.sv * pick(R.vars, q);
    double* sq = &s[q][0][0][0];
    constexpr int NL = (E3 + R3 - 1) / R3;
    double v[NL];
#pragma unroll
    for (int u = 0; u < NL; ++u) {  // every load in flight before the first store
      const int p = tid + u * R3;
      const int x = i0 + p % E, y = j0 + (p / E) % E, z = k0 + p / (E * E);
      if (p < E3 && x < g.ngi && y < g.ngj && z < g.ngk) v[u] = var[(long long)x + g.sy * y + g.sz * z];
    }
#pragma unroll
    for (int u = 0; u < NL; ++u) {
      const int p = tid + u * R3;
      const int x = i0 + p % E, y = j0 + (p / E) % E, z = k0 + p / (E * E);
      if (p < E3 && x < g.ngi && y < g.ngj && z < g.ngk) {
        sq[p] = v[u];
        if (unsafe_value(v[u], R.safe)) bits |= 1u << q;
      }
    }
  }
  __syncthreads();  // busy_s zeroed
  or_into(&busy_s, bits & cand & ((1u << R.nvars) - 1));
  __syncthreads();
  const unsigned busy = busy_s;
  if (!busy) return;
  if (tid <= W) {  // cells with x+y+z = w ordered by z then y
    int o = 0;
    for (int z = 0; z < T3; ++z)
      for (int w = 0; w < tid; ++w) o += row_cells(w - z);
    off[tid] = (short)o;
  }
  __syncthreads();
  for (int p = tid; p < C; p += R3) {
    const int x = p % T3, y = (p / T3) % T3, z = p / (T3 * T3), w = x + y + z;
    int r = off[w] + y - max(0, w - z - (T3 - 1));
    for (int zz = 0; zz < z; ++zz) r += row_cells(w - zz);
    order[r] = (unsigned short)p;
  }
  __syncthreads();
  const double D = R.dx * R.dx + R.dy * R.dy + R.dz * R.dz;
  const int q = tid >> 6, lt = tid & 63;  // this thread's variable and lane in its group
  const bool mine = q < R.nvars && ((busy >> q) & 1);
  for (int w = 0; w < W; ++w) {
    const int t = off[w] + lt;
    if (mine && t < off[w + 1]) {
      const int p = order[t];
      const int x = p % T3, y = (p / T3) % T3, z = p / (T3 * T3);
      if (x < xe && y < ye && z < ze) {
        double (*sv3)[E][E] = s[q];
        const int a = x + 1, b = y + 1, c = z + 1;
        const double nz = (double)((msk[p] >> q) & 1);
        const double lap = (sv3[c][b][a - 1] - 2 * sv3[c][b][a] + sv3[c][b][a + 1]) / (R.dx * R.dx) +
                           (sv3[c][b - 1][a] - 2 * sv3[c][b][a] + sv3[c][b + 1][a]) / (R.dy * R.dy) +
                           (sv3[c - 1][b][a] - 2 * sv3[c][b][a] + sv3[c + 1][b][a]) / (R.dz * R.dz);
        const double dnoise = R.eta * D * nz * lap;
        sv3[c][b][a] += dnoise;
      }
    }
    __syncthreads();
  }
  unsigned hard = 0;
  for (int qq = 0; qq < R.nvars; ++qq) {
    if (!((busy >> qq) & 1)) continue;
    double* var = U + g.sv * pick(R.vars, qq);
    for (int p = tid; p < C; p += R3) {
      const int x = p % T3, y = (p / T3) % T3, z = p / (T3 * T3);
      if (x < xe && y < ye && z < ze) {
        const double val = s[qq][z + 1][y + 1][x + 1];
        var[(long long)(i0 + 1 + x) + g.sy * (j0 + 1 + y) + g.sz * (k0 + 1 + z)] = val;
        if (hard_value(val, R.safe)) hard |= 1u << qq;
      }
    }
  }
  or_into(&hard_s, hard);
  __syncthreads();
  const unsigned hb = hard_s;
  if (hb && tid < 6) {  // mark the face neighbours for the variables left unsafe
    const int ax = tid >> 1, d = (tid & 1) ? 1 : -1;
    const int nx = tx + (ax == 0 ? d : 0), ny = ty + (ax == 1 ? d : 0), nz = tz + (ax == 2 ? d : 0);
    if (nx >= 0 && nx < ntx && ny >= 0 && ny < nty && nz >= 0 && nz < ntz)
      atomicOr(tiles + nx + ntx * (ny + nty * nz), (int)hb);
  }
}

// One diagonal (tx+ty = diag) of 32x32 interior tiles, one warp per filtered
// variable (at most two in 2D), swept side by side: lane t of warp q takes
// the t-th cell of variable q's wavefront w.
__global__ void __launch_bounds__(64) k_noise_remove2(Geo g, double* __restrict__ U,
                                                      const int* __restrict__ noise,
                                                      int* __restrict__ tiles, RemoveArgs R,
                                                      int diag, int ntx, int nty) {
  const int tx = blockIdx.x, ty = diag - tx;
  if (ty < 0 || ty >= nty) return;
  const unsigned cand = (unsigned)tiles[tx + ntx * ty];
  if (!cand) return;  // no variable to visit (k_noise_tiles2)
  constexpr int E = T2 + 2;
  __shared__ double s[2][E][E];  // per variable: [y][x]
  __shared__ int msk[T2 * T2];
  __shared__ unsigned busy_s, hard_s;
  const int tid = threadIdx.x;
  const int i0 = g.ng + T2 * tx - 1, j0 = g.ng + T2 * ty - 1;
  const int xe = min(T2, g.ngi - g.ng - (i0 + 1)), ye = min(T2, g.ngj - g.ng - (j0 + 1));
  if (tid == 0) busy_s = hard_s = 0;
  unsigned bits = 0;
  for (int p = tid; p < T2 * T2; p += 64) {
    const int x = p % T2, y = p / T2;
    const int m = x < xe && y < ye ? noise[(long long)(i0 + 1 + x) + g.sy * (j0 + 1 + y)] : 0;
    msk[p] = m;
    bits |= (unsigned)m;
  }
  for (int q = 0; q < R.nvars; ++q) {
    if (!((cand >> q) & 1)) continue;
    const double* var = U + g.sv * pick(R.vars, q);
    for (int p = tid; p < E * E; p += 64) {
      const int a = p % E, b = p / E;
      const int x = i0 + a, y = j0 + b;
      if (x < g.ngi && y < g.ngj) {
        const double val = var[(long long)x + g.sy * y];
        s[q][b][a] = val;
        if (unsafe_value(val, R.safe)) bits |= 1u << q;
      }
    }
  }
  __syncthreads();
  or_into(&busy_s, bits & cand & ((1u << R.nvars) - 1));
  __syncthreads();
  const unsigned busy = busy_s;
  if (!busy) return;
  const double dx = R.dx, dy = R.dy;
  const double D = dx * dx + dy * dy;
  const int q = tid >> 5, lt = tid & 31;
  const bool mine = q < R.nvars && ((busy >> q) & 1);
  for (int w = 0; w < 2 * T2 - 1; ++w) {
    const int y = max(0, w - (T2 - 1)) + lt, x = w - y;  // x >= 0 while y <= w
    if (mine && x >= 0 && y < ye && x < xe) {
      const int a = x + 1, b = y + 1;
      const double nz = (double)((msk[x + T2 * y] >> q) & 1);
      const double lgrad = (s[q][b][a] - s[q][b][a - 1]) / dx;
      const double rgrad = (s[q][b][a + 1] - s[q][b][a]) / dx;
      const double bgrad = (s[q][b][a] - s[q][b - 1][a]) / dy;
      const double tgrad = (s[q][b + 1][a] - s[q][b][a]) / dy;
      const double dv = R.eta * D * nz * ((rgrad - lgrad) / dx + (tgrad - bgrad) / dy);
      s[q][b][a] += dv;
    }
    __syncwarp();  // each variable's steps stay within its own warp
  }
  __syncthreads();
  unsigned hard = 0;
  for (int qq = 0; qq < R.nvars; ++qq) {
    if (!((busy >> qq) & 1)) continue;
    double* var = U + g.sv * pick(R.vars, qq);
    for (int p = tid; p < T2 * T2; p += 64) {
      const int x = p % T2, y = p / T2;
      if (x < xe && y < ye) {
        const double val = s[qq][y + 1][x + 1];
        var[(long long)(i0 + 1 + x) + g.sy * (j0 + 1 + y)] = val;
        if (hard_value(val, R.safe)) hard |= 1u << qq;
      }
    }
  }
  or_into(&hard_s, hard);
  __syncthreads();
  const unsigned hb = hard_s;
  if (hb && tid < 4) {  // mark the face neighbours
    const int d = (tid & 1) ? 1 : -1;
    const int nx = tx + (tid < 2 ? d : 0), ny = ty + (tid < 2 ? 0 : d);
    if (nx >= 0 && nx < ntx && ny >= 0 && ny < nty) atomicOr(tiles + nx + ntx * ny, (int)hb);
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

long long fst_noise_ints(const Geo& g) {
  const long long tiles = g.ndim == 3 ? (long long)((g.nci + T3 - 1) / T3) * ((g.ncj + T3 - 1) / T3) *
                                            ((g.nck + T3 - 1) / T3)
                                      : (long long)((g.nci + T2 - 1) / T2) * ((g.ncj + T2 - 1) / T2);
  return g.sv + tiles;
}

void fst_noise_graph_release(NoiseGraph& ng) {
  if (ng.exec) cudaGraphExecDestroy(ng.exec);
  if (ng.cap) cudaStreamDestroy(ng.cap);
  ng = NoiseGraph{};
}

int fst_noise_launch(const Geo& g, const fst_config& cf, double* U, int* noise,
                     unsigned long long* key, const fst_noise_params& np, cudaStream_t st,
                     Prof* prof, NoiseGraph* graph) {
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
    fst_fill_keys(key, 1, FST_KEY_LOWEST, st);
    // 3D: maxCvar3D(var, 6), a fixed index (src/cart3d.cpp:346); 2D: C_hat
    const int cv = g.ndim == 3 ? 6 : g.nv + 1;
    FST_LAUNCH(prof, "noise_max", st, n, k_noise_maxabs<<<8 * 152, 256, 0, st>>>(g, U, cv, key));
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
  int* tiles = noise + g.sv;  // candidate tiles (fst_noise_ints)
  // the tile marks, then nt sweeps of one launch per tile diagonal
  auto sweeps = [&](cudaStream_t s, Prof* pr) {
    int L = 0;
    if (g.ndim == 3) {
      const int ntx = (g.nci + T3 - 1) / T3, nty = (g.ncj + T3 - 1) / T3, ntz = (g.nck + T3 - 1) / T3;
      FST_LAUNCH(pr, "noise_tiles", s, L,
                 k_noise_tiles3<<<ntx * nty * ntz, 256, 0, s>>>(g, U, noise, tiles, R, ntx, nty));
      for (int tau = 0; tau < np.nt; ++tau)
        for (int d = 0; d <= ntx + nty + ntz - 3; ++d)
          FST_LAUNCH(pr, "noise_remove", s, L,
                     k_noise_remove3<<<ntx * nty, R3, 0, s>>>(g, U, noise, tiles, R, d, ntx, nty, ntz));
    } else {
      const int ntx = (g.nci + T2 - 1) / T2, nty = (g.ncj + T2 - 1) / T2;
      FST_LAUNCH(pr, "noise_tiles", s, L,
                 k_noise_tiles2<<<ntx * nty, 256, 0, s>>>(g, U, noise, tiles, R, ntx));
      for (int tau = 0; tau < np.nt; ++tau)
        for (int d = 0; d <= ntx + nty - 2; ++d)
          FST_LAUNCH(pr, "noise_remove", s, L,
                     k_noise_remove2<<<ntx, 64, 0, s>>>(g, U, noise, tiles, R, d, ntx, nty));
    }
    return L;
  };
  if (np.nt <= 0) return n;
  if (!graph || (prof && prof->on)) return n + sweeps(st, prof);  // per-kernel timing
  // the launch parameters the graph bakes in
  struct Sig {
    const double* U;
    const int* noise;
    RemoveArgs R;
    int nt, ndim, nci, ncj, nck;
  } sig;
  memset(&sig, 0, sizeof(sig));
  sig.U = U;
  sig.noise = noise;
  sig.R = R;
  sig.nt = np.nt;
  sig.ndim = g.ndim;
  sig.nci = g.nci;
  sig.ncj = g.ncj;
  sig.nck = g.nck;
  static_assert(sizeof(Sig) <= sizeof(graph->sig), "noise graph signature");
  if (!graph->exec || memcmp(graph->sig, &sig, sizeof(sig)) != 0) {
    if (graph->exec) cudaGraphExecDestroy(graph->exec);
    graph->exec = nullptr;
    cudaError_t e = cudaSuccess;
    if (!graph->cap) e = cudaStreamCreateWithFlags(&graph->cap, cudaStreamNonBlocking);
    cudaGraph_t gr = nullptr;
    if (e == cudaSuccess) e = cudaStreamBeginCapture(graph->cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      graph->launches = sweeps(graph->cap, nullptr);
      e = cudaStreamEndCapture(graph->cap, &gr);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&graph->exec, gr, 0);
    if (gr) cudaGraphDestroy(gr);
    if (e != cudaSuccess) {  // no graph on this setup: launch the sweeps directly
      if (graph->exec) cudaGraphExecDestroy(graph->exec);
      graph->exec = nullptr;
      cudaGetLastError();
      return n + sweeps(st, prof);
    }
    memcpy(graph->sig, &sig, sizeof(sig));
  }
  cudaGraphLaunch(graph->exec, st);
  return n + graph->launches;
}
