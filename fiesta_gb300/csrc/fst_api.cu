// fst_api.cu — the libfst C ABI (include/fst.h): context lifetime, state
// transfer, and the per-step sequencing that replaces rkAdvance
// (src/rk.cpp:28-70) with its calls into cart3d_func / cart2d_func::compute.
//
// State lives in two device buffers A and B.  Stage 1 reads A, writes
// B = A + (0.5*dt)*R(A); stage 2 reads B and writes A = A + dt*R(B) in place
// (each cell reads only its own old value).  This replaces the reference's
// tmp1 copy and its separate dvar array: the stage combine is fused into the
// cell kernel and R never goes to HBM.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>  // header-only; ranges are no-ops without a tool attached

#include "fst_common.cuh"
#include "fst_internal.h"

namespace {

DivC make_div(double d) {
  DivC q;
  q.d = d;
  int e = 0;
  double m = std::frexp(d, &e);
  q.inv = (d > 0.0 && m == 0.5 && std::isfinite(1.0 / d)) ? 1.0 / d : 0.0;
  return q;
}

bool bc_ok(int t) { return t >= FST_BC_OUTFLOW && t <= FST_BC_HYDROSTATIC; }

}  // namespace

struct fst_ctx {
  fst_config cf;
  Geo g;
  Phys P;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  double* Ua = nullptr;
  double* Ub = nullptr;
  double* Rdev = nullptr;  // compute_rhs output (zero outside the interior)
  Plain3DBufs b3{};
  Plain2DBufs b2{};
  MixedBufs bm{};
  std::vector<void*> allocs;
  std::vector<size_t> alloc_bytes;
  std::string err;
  unsigned long long* dstat = nullptr;  // fst_status keys
  int* dnoise = nullptr;                 // noise indicator (fst_noise_filter)
  unsigned long long* dnoise_key = nullptr;
  NoiseGraph noise_graph;                // the filter's sweeps as a CUDA graph
  fst_stats stats{};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool timed = false;
  // fst_rk_step_get_state: the side stream of the overlapped download
  MixedDownload dl{};
  int* dflag = nullptr;
  bool gen = false;       // FST_GRID_GENERALIZED
  bool grid_set = false;  // fst_set_grid has computed the metrics
  Prof prof;
};

namespace {

int fail(fst_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(fst_ctx* c, cudaError_t e, const char* what) {
  return fail(c, FST_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int check_launch(fst_ctx* c, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, what);
  return FST_OK;
}

// Reads FST_MAX_DEVICE_BYTES: an artificial device-memory limit used to
// exercise the out-of-memory path without exhausting a GPU.
size_t device_limit() {
  const char* s = std::getenv("FST_MAX_DEVICE_BYTES");
  if (!s || !*s) return (size_t)-1;
  return (size_t)std::strtoull(s, nullptr, 10);
}

std::string validate(const fst_config* cf) {
  if (cf->abi_version != FST_ABI_VERSION) return "abi_version mismatch";
  if (cf->ndim != 2 && cf->ndim != 3) return "ndim must be 2 or 3";
  if (cf->ng != 3) return "ng must be 3 (the WENO5 stencil needs three ghost layers)";
  if (cf->nci < 1 || cf->ncj < 1 || (cf->ndim == 3 && cf->nck < 1)) return "grid sizes must be >= 1";
  if (cf->ns < 1 || cf->ns > FST_MAX_SPECIES) return "ns must be in [1, 16]";
  if (!(cf->dx > 0) || !(cf->dy > 0) || (cf->ndim == 3 && !(cf->dz > 0)))
    return "cell sizes must be positive";
  if (!std::isfinite(cf->dt)) return "dt must be finite";
  for (int s = 0; s < cf->ns; ++s) {
    if (!(cf->gamma[s] > 1.0)) return "species gamma must be > 1";
    if (!(cf->M[s] > 0.0)) return "species molar mass must be > 0";
  }
  const int b[6] = {cf->bc_xmin, cf->bc_xmax, cf->bc_ymin, cf->bc_ymax, cf->bc_zmin, cf->bc_zmax};
  for (int q = 0; q < 6; ++q)
    if (!bc_ok(b[q])) return "unknown boundary condition type";
  if (cf->mode < FST_MODE_PLAIN_FP64 || cf->mode > FST_MODE_HYBRID) return "unknown mode";
  if (cf->audit_every < 0 || cf->classify_every < 0) return "negative audit / classify period";
  if (cf->grid_type != FST_GRID_CARTESIAN && cf->grid_type != FST_GRID_GENERALIZED)
    return "unknown grid type";
  if (cf->scheme < 0 || cf->scheme > FST_SCHEME_QUICK) return "unknown advection scheme";
  if (cf->ndim == 2 && cf->scheme > FST_SCHEME_WENO5 && cf->mode != FST_MODE_PLAIN_FP64)
    return "the centered4 and quick schemes run in FST_MODE_PLAIN_FP64";
  if (cf->grid_type == FST_GRID_GENERALIZED) {
    if (cf->mode == FST_MODE_HYBRID || (cf->mode == FST_MODE_MIXED && cf->ndim != 3))
      return "generalized grids run in FST_MODE_PLAIN_FP64 (and FST_MODE_MIXED in 3D)";
    // the reference's gen2d / gen3d modules exchange no halo and apply no
    // boundary conditions, so a periodic axis has no meaning there
    if (cf->xper || cf->yper || (cf->ndim == 3 && cf->zper))
      return "periodic axes are not supported on generalized grids";
  }
  long long ngi = cf->nci + 6LL, ngj = cf->ncj + 6LL, ngk = cf->ndim == 3 ? cf->nck + 6LL : 1;
  if (ngi * ngj * ngk > (1LL << 40)) return "grid too large";
  return "";
}

void setup_phys(const fst_config& cf, const Geo& g, Phys& P) {
  std::memset(&P, 0, sizeof(P));
  P.ns = g.ns;
  P.nv = g.nv;
  P.nvt = g.nvt;
  // gen2d / gen3d compute advection and the pressure gradient only
  const bool cart = cf.grid_type != FST_GRID_GENERALIZED;
  P.visc = cart && cf.visc != 0;
  P.ceq = cart && cf.ceq != 0;
  P.buoyancy = cart && cf.buoyancy != 0;
  P.scheme = g.ndim == 2 && cf.scheme > 0 ? cf.scheme : FST_SCHEME_WENO5;
  // device config array of the reference (src/cart3d.cpp:152-171)
  std::vector<double> cd(6 + 3 * g.ns, 0.0);
  for (int s = 0; s < g.ns; ++s) {
    cd[6 + 3 * s] = cf.gamma[s];
    cd[7 + 3 * s] = cf.R / cf.M[s];
    cd[8 + 3 * s] = cf.mu[s];
  }
  for (int s = 0; s < g.ns; ++s) {
    double gs = cd[6 + 3 * s], Rs = cd[7 + 3 * s];
    P.cp_s[s] = gs * Rs / (gs - 1);
    P.cv_s[s] = Rs / (gs - 1);
    P.mu_s[s] = cd[8 + 3 * s];
    double g2 = cd[6 + 2 * s], R2 = cd[6 + 2 * s + 1];
    P.cp2_s[s] = g2 * R2 / (g2 - 1);
    P.cv2_s[s] = R2 / (g2 - 1);
  }
  P.dx = cf.dx;
  P.dy = cf.dy;
  // 2D: dz = dx (src/input.cpp:402); the generalized 3D module passes cf.dx as
  // the z spacing of its fluxes (src/gen3d.cpp:359), its only use of dz
  P.dz = g.ndim == 3 && cart ? cf.dz : cf.dx;
  P.ddx = make_div(P.dx);
  P.ddy = make_div(P.dy);
  P.ddz = make_div(P.dz);
  P.d4x = make_div(4 * P.dx);
  P.d4y = make_div(4 * P.dy);
  P.d4z = make_div(4 * P.dz);
  P.d12x = 12.0 * P.dx;
  P.d12y = 12.0 * P.dy;
  P.d12z = 12.0 * P.dz;
  P.d12pz = 12.0 * P.dy;
  P.r12x = 1.0 / P.d12x;
  P.r12y = 1.0 / P.d12y;
  P.r12pz = 1.0 / P.d12pz;
  P.dt = cf.dt;
  P.hdt = 0.5f * cf.dt;
  P.kap = cf.kap;
  P.eps = cf.eps;
  P.alpha = cf.alpha;
  P.g = cf.g_accel;
  P.rho_ref = cf.rho_ref;
  if (g.ndim == 3) {
    P.dxmag2 = P.dx * P.dx + P.dy * P.dy + P.dz * P.dz;
    P.dxmag = std::sqrt(P.dx * P.dx + P.dy * P.dy + P.dz * P.dz);
  } else {
    P.dxmag2 = P.dx * P.dx + P.dy * P.dy;
    P.dxmag = std::sqrt(P.dx * P.dx + P.dy * P.dy);
  }
  P.mu2d = 2.928e-5;
  P.kheat2d = 0.026;
  P.rd_f[0] = (float)(1.0 / P.dx);
  P.rd_f[1] = (float)(1.0 / P.dy);
  P.rd_f[2] = (float)(1.0 / P.dz);
  P.r12_f[0] = (float)(1.0 / P.d12x);
  P.r12_f[1] = (float)(1.0 / P.d12y);
  P.r12_f[2] = (float)(1.0 / P.d12z);
  P.dxmag_f = (float)P.dxmag;
  P.dxmag2_f = (float)P.dxmag2;
  P.eps_f = (float)P.eps;
  P.kap_f = (float)P.kap;
  P.alpha_f = (float)P.alpha;
  P.mu2d_f = (float)P.mu2d;
  P.kheat_f = (float)P.kheat2d;
  for (int s = 0; s < g.ns; ++s) {
    P.rm_s[s] = P.cp_s[s] - P.cv_s[s];
    P.cv_f[s] = (float)P.cv_s[s];
    P.rm_f[s] = (float)(P.cp_s[s] - P.cv_s[s]);
    P.cv_lf[s] = (float)(P.cv_s[s] - (double)P.cv_f[s]);
    P.rm_lf[s] = (float)(P.rm_s[s] - (double)P.rm_f[s]);
    P.mu_f[s] = (float)P.mu_s[s];
    P.cv2_f[s] = (float)P.cv2_s[s];
    P.cp2_f[s] = (float)P.cp2_s[s];
  }
}

// Device bytes of the work arrays of each path, in doubles per cell.
size_t work_doubles_per_cell(const fst_config& cf, const Geo& g) {
  size_t w = 0;
  const bool gen = cf.grid_type == FST_GRID_GENERALIZED;
  const bool visc = cf.visc && !gen, ceq = cf.ceq && !gen;
  if (cf.mode == FST_MODE_PLAIN_FP64) {
    if (g.ndim == 3) {
      w = 2 + 3 + 1 + 1 + (size_t)3 * g.nv;  // rho p vel T nrg F
      if (visc) w += g.ns + 18;
      if (ceq) w += 27;
      if (gen) w += 9;
    } else {
      w = 2 + 2 + 1 + 1 + (size_t)2 * g.nv;
      if (visc) w += 6 + 2;
      if (ceq) w += 8;
      if (gen) w += 4;
    }
  } else {
    w = fst_mixed_work_doubles_per_cell(cf, g);
  }
  return w;
}

// FP64 FMA throughput: 8 independent FMA chains per thread, every SM full.
__global__ void __launch_bounds__(256) k_fp64_rate(double* __restrict__ out, int iters) {
  double a[8];
  const double x = 1.0 + 1e-9 * threadIdx.x, y = 1.0 - 1e-9 * blockIdx.x;
#pragma unroll
  for (int q = 0; q < 8; ++q) a[q] = q;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int q = 0; q < 8; ++q) a[q] = fma(a[q], x, y);
  }
  double sum = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) sum += a[q];
  if (sum == 12345.678) out[0] = sum;  // keeps the chains live
}

__global__ void k_nonfinite(const double* __restrict__ U, long long n, int* flag) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; t < n; t += (long long)gridDim.x * blockDim.x)
    if (!isfinite(U[t])) {
      *flag = 1;
      return;
    }
}

// Per-field minimum and maximum over the interior, as statusCheck's Max/Min
// reductions (src/status.cpp:86-99, 155-235): strict comparisons against
// the identities -DBL_MAX / +DBL_MAX, so NaN never enters and -inf (+inf)
// never becomes a maximum (minimum).  Keys: [2f] max, [2f+1] max of -x.
struct StatusFields {
  const double* f[FST_MAXV + 6];
};
__global__ void __launch_bounds__(256) k_status(Geo g, StatusFields F,
                                                unsigned long long* __restrict__ keys) {
  const double* a = F.f[blockIdx.y];
  const int rows = g.ncj * (g.ndim == 3 ? g.nck : 1);
  // per-thread extremes on the order-preserving integer key: FP64 compares
  // would run on the FP64 pipe, two per value; NaN is skipped, as by the
  // reference's `if (v > max)` reducers
  unsigned long long kmx = FST_KEY_LOWEST, kmn = 0xFFEFFFFFFFFFFFFFull;  // keys of -+DBL_MAX
  constexpr int RB = 8;  // interior rows per step, their loads in flight together
  for (int r0 = blockIdx.x * RB; r0 < rows; r0 += gridDim.x * RB)
    for (int i = threadIdx.x; i < g.nci; i += 256) {
      unsigned long long v[RB];
#pragma unroll
      for (int u = 0; u < RB; ++u) {
        const int r = r0 + u < rows ? r0 + u : 0, j = r % g.ncj, k = r / g.ncj;  // past the end: row 0
        v[u] = fst_bits(a[g.ng + i + g.sy * (j + g.ng) + g.sz * (g.ndim == 3 ? k + g.ng : 0)]);
      }
#pragma unroll
      for (int u = 0; u < RB; ++u) {
        if ((v[u] & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull) continue;  // NaN
        const unsigned long long key = (v[u] >> 63) ? ~v[u] : (v[u] | 0x8000000000000000ull);
        kmx = key > kmx ? key : kmx;
        kmn = key < kmn ? key : kmn;
      }
    }
  double mx = fst_unkey(kmx), mn = fst_unkey(kmn);
  __shared__ double smx[8], smn[8];
  mx = fst_warp_max(mx);
  mn = -fst_warp_max(-mn);
  if ((threadIdx.x & 31) == 0) {
    smx[threadIdx.x >> 5] = mx;
    smn[threadIdx.x >> 5] = mn;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) {
      if (smx[w] > mx) mx = smx[w];
      if (smn[w] < mn) mn = smn[w];
    }
    atomicMax(&keys[2 * blockIdx.y], fst_key(mx));
    atomicMax(&keys[2 * blockIdx.y + 1], fst_key(-mn));
  }
}

int alloc(fst_ctx* c, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, FST_ERR_OOM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
  }
  c->allocs.push_back(*p);
  c->alloc_bytes.push_back(bytes);
  return FST_OK;
}

template <class T>
int allocd(fst_ctx* c, T** p, size_t n) {
  return alloc(c, (void**)p, n * sizeof(T));
}

int stage(fst_ctx* c, const double* Uin, const double* Uold, double* Unew, double coef,
          double* Rout, bool ghosts) {
  nvtxRangePushA(Rout ? "fst rhs" : "fst rk stage");
  int n;
  if (c->cf.mode != FST_MODE_PLAIN_FP64)
    n = fst_mixed_stage(c->g, c->P, c->cf, c->bm, Uin, Uold, Unew, coef, Rout, ghosts, c->stream,
                        &c->prof);
  else if (c->g.ndim == 3)
    n = fst_plain3d_stage(c->g, c->P, c->b3, Uin, Uold, Unew, coef, Rout, ghosts, c->stream,
                          &c->prof);
  else
    n = fst_plain2d_stage(c->g, c->P, c->b2, Uin, Uold, Unew, coef, Rout, ghosts, c->stream,
                          &c->prof);
  c->stats.kernel_launches += n;
  nvtxRangePop();
  return check_launch(c, "stage kernels");
}

int bcs(fst_ctx* c, double* U) {
  c->stats.kernel_launches += fst_launch_bcs(c->g, c->cf, U, c->stream, &c->prof);
  return check_launch(c, "boundary kernels");
}

}  // namespace

// Geometry and physics constants of a config, for entry points that run
// without a context (fst_noalloc.cu).  Returns "" or the validation error.
std::string fst_setup_geo_phys(const fst_config* cfg, Geo& g, Phys& P) {
  std::string why = validate(cfg);
  if (!why.empty()) return why;
  g.ndim = cfg->ndim;
  g.ng = cfg->ng;
  g.nci = cfg->nci;
  g.ncj = cfg->ncj;
  g.nck = g.ndim == 3 ? cfg->nck : 1;
  g.ngi = g.nci + 2 * g.ng;
  g.ngj = g.ncj + 2 * g.ng;
  g.ngk = g.ndim == 3 ? g.nck + 2 * g.ng : 1;
  g.ns = cfg->ns;
  g.nv = (g.ndim == 3 ? 4 : 3) + g.ns;
  g.nvt = g.nv + (cfg->ceq ? 5 : 0);
  g.sy = g.ngi;
  g.sz = (long long)g.ngi * g.ngj;
  g.sv = g.sz * g.ngk;
  setup_phys(*cfg, g, P);
  return "";
}

// After a synchronisation: the device error word of the 3D mixed kernels
// (a TMA wait that ran out), cleared once reported.
int device_errors(fst_ctx* c) {
  if (!c->bm.dev_err) return FST_OK;
  unsigned int h = 0;
  cudaError_t e = cudaMemcpy(&h, c->bm.dev_err, sizeof(h), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(c, e, "device error word");
  if (!h) return FST_OK;
  cudaMemset(c->bm.dev_err, 0, sizeof(h));
  return fail(c, FST_ERR_TIMEOUT, "a shared-memory plane load did not complete in time");
}

extern "C" {

const char* fst_last_error(const fst_ctx* c) { return c ? c->err.c_str() : "null context"; }

int fst_create(const fst_config* cfg, fst_ctx** out) {
  if (!cfg || !out) return FST_ERR_INVALID;
  *out = nullptr;
  std::string why = validate(cfg);
  if (!why.empty()) {
    std::fprintf(stderr, "fst_create: %s\n", why.c_str());
    return FST_ERR_INVALID;
  }
  fst_ctx* c = new fst_ctx();
  c->cf = *cfg;
  Geo& g = c->g;
  g.ndim = cfg->ndim;
  g.ng = cfg->ng;
  g.nci = cfg->nci;
  g.ncj = cfg->ncj;
  g.nck = g.ndim == 3 ? cfg->nck : 1;
  g.ngi = g.nci + 2 * g.ng;
  g.ngj = g.ncj + 2 * g.ng;
  g.ngk = g.ndim == 3 ? g.nck + 2 * g.ng : 1;
  g.ns = cfg->ns;
  g.nv = (g.ndim == 3 ? 4 : 3) + g.ns;
  g.nvt = g.nv + (cfg->ceq ? 5 : 0);
  g.sy = g.ngi;
  g.sz = (long long)g.ngi * g.ngj;
  g.sv = g.sz * g.ngk;
  setup_phys(*cfg, g, c->P);

  const size_t cells = (size_t)g.sv;
  const size_t need = cells * sizeof(double) * (2 * (size_t)g.nvt + work_doubles_per_cell(*cfg, g));
  if (need > device_limit()) {
    std::fprintf(stderr, "fst_create: %zu device bytes over the FST_MAX_DEVICE_BYTES limit\n", need);
    delete c;
    return FST_ERR_OOM;
  }
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "fst_create: no CUDA device: %s\n", cudaGetErrorString(e));
    cudaGetLastError();
    delete c;
    return FST_ERR_CUDA;
  }
  int rc = FST_OK;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) rc = cuda_fail(c, e, "cudaStreamCreate");
  c->own_stream = true;
  const size_t nst = cells * g.nvt;
  if (!rc) rc = allocd(c, &c->Ua, nst);
  if (!rc) rc = allocd(c, &c->Ub, nst);
  if (!rc) rc = allocd(c, &c->dflag, 1);
  c->gen = cfg->grid_type == FST_GRID_GENERALIZED;
  if (!rc && cfg->mode == FST_MODE_PLAIN_FP64 && g.ndim == 3) {
    Plain3DBufs& b = c->b3;
    rc = allocd(c, &b.rho, cells);
    if (!rc) rc = allocd(c, &b.pr, cells);
    if (!rc) rc = allocd(c, &b.vel, 3 * cells);
    if (!rc) rc = allocd(c, &b.T, cells);
    if (!rc) rc = allocd(c, &b.nrg, cells);
    if (!rc) rc = allocd(c, &b.F, (size_t)3 * g.nv * cells);
    if (!rc && c->P.visc) rc = allocd(c, &b.Y, (size_t)g.ns * cells);
    if (!rc && c->P.visc) rc = allocd(c, &b.S, 18 * cells);
    if (!rc && c->P.ceq) rc = allocd(c, &b.MF, 27 * cells);
    if (!rc && c->gen) rc = allocd(c, &b.met, 9 * cells);
    if (!rc) rc = allocd(c, &b.red, 2);
  } else if (!rc && cfg->mode == FST_MODE_PLAIN_FP64) {
    Plain2DBufs& b = c->b2;
    rc = allocd(c, &b.rho, cells);
    if (!rc) rc = allocd(c, &b.pr, cells);
    if (!rc) rc = allocd(c, &b.vel, 2 * cells);
    if (!rc) rc = allocd(c, &b.T, cells);
    if (!rc) rc = allocd(c, &b.nrg, cells);
    if (!rc) rc = allocd(c, &b.F, (size_t)2 * g.nv * cells);
    if (!rc && c->P.visc) rc = allocd(c, &b.S, 6 * cells);
    if (!rc && c->P.visc) rc = allocd(c, &b.Q, 2 * cells);
    if (!rc && c->P.ceq) rc = allocd(c, &b.MF, 8 * cells);
    if (!rc && c->gen) rc = allocd(c, &b.met, 4 * cells);
    if (!rc) rc = allocd(c, &b.red, 2);
  } else if (!rc) {
    std::string why;
    rc = fst_mixed_alloc(*cfg, g, c->bm, [&](void** p, size_t bytes) { return alloc(c, p, bytes); },
                         &why);
    if (rc && !why.empty()) fail(c, rc, why);
  }
  // zero state like a fresh Kokkos View; zero work arrays so that entries
  // outside each kernel's range read as the reference's zero-initialised ones
  if (!rc) {
    for (size_t q = 0; q < c->alloc_bytes.size() && e == cudaSuccess; ++q)
      e = cudaMemsetAsync(c->allocs[q], 0, c->alloc_bytes[q], c->stream);
    if (e != cudaSuccess) rc = cuda_fail(c, e, "cudaMemset");
  }
  // FST_DEBUG_CANARY=1: the mixed path's primitive arrays start as NaN, so a
  // read of an entry no kernel writes (row padding, halo beyond the grid)
  // that reached an output would show up (tests compare against a normal run)
  if (!rc && cfg->mode != FST_MODE_PLAIN_FP64) {
    const char* cv = std::getenv("FST_DEBUG_CANARY");
    if (cv && *cv == '1') {
      e = fst_mixed_canary(g, c->bm, c->stream);
      if (e != cudaSuccess) rc = cuda_fail(c, e, "canary fill");
    }
  }
  if (!rc) {
    e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e != cudaSuccess) rc = cuda_fail(c, e, "cudaEventCreate");
  }
  if (!rc) {
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = cuda_fail(c, e, "create sync");
  }
  if (rc) {
    std::fprintf(stderr, "fst_create: %s\n", c->err.c_str());
    fst_destroy(c);
    return rc;
  }
  *out = c;
  return FST_OK;
}

void fst_destroy(fst_ctx* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (void* p : c->allocs) cudaFree(p);
  fst_mixed3d_release(c->bm);
  fst_noise_graph_release(c->noise_graph);
  if (c->Rdev) cudaFree(c->Rdev);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->dl.side) {
    cudaStreamSynchronize(c->dl.side);
    cudaStreamDestroy(c->dl.side);
    for (cudaEvent_t e : c->dl.ev) cudaEventDestroy(e);
  }
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int fst_set_stream(fst_ctx* c, void* s) {
  if (!c) return FST_ERR_INVALID;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "set_stream sync");
  if (c->own_stream) cudaStreamDestroy(c->stream);
  c->own_stream = false;
  c->stream = (cudaStream_t)s;
  return FST_OK;
}

int fst_synchronize(fst_ctx* c) {
  if (!c) return FST_ERR_INVALID;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "synchronize");
  return device_errors(c);
}

namespace {
// A device-visible address of host buffer U[0..n) for a kernel to read, or
// null: both ends page-locked (cudaHostAlloc / cudaHostRegister) with
// consistent device addresses, on a device that can also reach pageable
// memory (so no address in between can fault).
const double* device_view_of_host(const double* U, size_t n, int dev) {
  int pageable = 0;
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (!pageable || n == 0) return nullptr;
  cudaPointerAttributes a0{}, a1{};
  if (cudaPointerGetAttributes(&a0, U) != cudaSuccess ||
      cudaPointerGetAttributes(&a1, U + (n - 1)) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer ||
      !a1.devicePointer)
    return nullptr;
  const double* d0 = static_cast<const double*>(a0.devicePointer);
  if (static_cast<const double*>(a1.devicePointer) != d0 + (n - 1)) return nullptr;
  return d0;
}
}  // namespace

int fst_set_state(fst_ctx* c, const double* U, size_t n) {
  if (!c || !U) return FST_ERR_INVALID;
  if (n != (size_t)c->g.sv * c->g.nvt) return fail(c, FST_ERR_SIZE, "state size mismatch");
  c->bm.fused_for = nullptr;  // the primitives no longer describe the state
  if (c->cf.mode != FST_MODE_PLAIN_FP64 && c->bm.fused && !c->gen &&
      !std::getenv("FST_NO_FUSED_UPLOAD")) {
    if (const double* Ud = device_view_of_host(U, n, c->device)) {
      const int k = fst_mixed_upload(c->g, c->P, c->bm, Ud, c->Ua, c->stream, &c->prof);
      if (k >= 0) {
        c->stats.kernel_launches += k;
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) {
          c->bm.fused_for = nullptr;
          return cuda_fail(c, e, "set_state (fused upload)");
        }
        return FST_OK;
      }
    }
  }
  cudaError_t e = cudaMemcpyAsync(c->Ua, U, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "set_state");
  return FST_OK;
}

int fst_get_state(fst_ctx* c, double* U, size_t n) {
  if (!c || !U) return FST_ERR_INVALID;
  if (n != (size_t)c->g.sv * c->g.nvt) return fail(c, FST_ERR_SIZE, "state size mismatch");
  cudaError_t e = cudaMemcpyAsync(U, c->Ua, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "get_state");
  return device_errors(c);
}

int fst_set_state_device(fst_ctx* c, const double* dU, size_t n) {
  if (!c || !dU) return FST_ERR_INVALID;
  if (n != (size_t)c->g.sv * c->g.nvt) return fail(c, FST_ERR_SIZE, "state size mismatch");
  c->bm.fused_for = nullptr;
  cudaError_t e = cudaMemcpyAsync(c->Ua, dU, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "set_state_device");
  return FST_OK;
}

int fst_get_state_device(fst_ctx* c, double* dU, size_t n) {
  if (!c || !dU) return FST_ERR_INVALID;
  if (n != (size_t)c->g.sv * c->g.nvt) return fail(c, FST_ERR_SIZE, "state size mismatch");
  cudaError_t e = cudaMemcpyAsync(dU, c->Ua, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "get_state_device");
  return FST_OK;
}

int fst_apply_bcs(fst_ctx* c) {
  if (!c) return FST_ERR_INVALID;
  return bcs(c, c->Ua);
}

int fst_compute_rhs(fst_ctx* c, double* R, size_t n) {
  if (!c) return FST_ERR_INVALID;
  const size_t nst = (size_t)c->g.sv * c->g.nvt;
  if (R && n != nst) return fail(c, FST_ERR_SIZE, "rhs size mismatch");
  if (!c->Rdev) {
    cudaError_t e = cudaMalloc(&c->Rdev, nst * sizeof(double));
    if (e != cudaSuccess) {
      c->Rdev = nullptr;
      cudaGetLastError();
      return fail(c, FST_ERR_OOM, "rhs buffer allocation failed");
    }
    e = cudaMemsetAsync(c->Rdev, 0, nst * sizeof(double), c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "rhs memset");
  }
  if (c->gen && !c->grid_set) return fail(c, FST_ERR_INVALID, "fst_set_grid has not been called");
  int rc = FST_OK;
  if (c->g.ndim == 3 && !c->gen) rc = bcs(c, c->Ua);  // cart3d_func::compute applies BCs first
  c->bm.stage = 0;
  c->bm.classified = false;
  if (!rc) rc = stage(c, c->Ua, c->Ua, nullptr, 0.0, c->Rdev, false);
  if (rc) return rc;
  if (R) {
    cudaError_t e = cudaMemcpyAsync(R, c->Rdev, nst * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "compute_rhs copy");
  }
  return FST_OK;
}

namespace {
// One time step: preStep (BCs on cartesian grids), stage 1 into Ub (ghosts
// copied), BCs on Ub (3D cartesian), stage 2 into Ua.  A download plan in
// c->bm.dl applies to stage 2 only.
int one_step(fst_ctx* c) {
  int rc = FST_OK;
  const bool two_d = c->g.ndim == 2;
  // gen2d / gen3d apply no boundary conditions (src/gen2d.cpp:132-134,
  // src/gen3d.cpp:109, 338-370)
  if (two_d && !c->gen) rc = bcs(c, c->Ua);  // cart2d_func::preStep
  if (!rc && !two_d && !c->gen) rc = bcs(c, c->Ua);
  c->bm.stage = 1;
  MixedDownload* dl = c->bm.dl;
  c->bm.dl = nullptr;
  if (!rc) rc = stage(c, c->Ua, c->Ua, c->Ub, c->P.hdt, nullptr, true);
  c->bm.dl = dl;
  if (!rc && !two_d && !c->gen) rc = bcs(c, c->Ub);
  c->bm.stage = 2;
  if (!rc) rc = stage(c, c->Ub, c->Ua, c->Ua, c->P.dt, nullptr, false);
  if (rc) return rc;
  c->bm.step += 1;
  c->stats.steps += 1;
  return FST_OK;
}
}  // namespace

int fst_rk_step(fst_ctx* c, int nsteps) {
  if (!c || nsteps < 0) return FST_ERR_INVALID;
  if (c->gen && !c->grid_set) return fail(c, FST_ERR_INVALID, "fst_set_grid has not been called");
  cudaEventRecord(c->ev0, c->stream);
  for (int s = 0; s < nsteps; ++s) {
    const int rc = one_step(c);
    if (rc) return rc;
  }
  cudaEventRecord(c->ev1, c->stream);
  c->timed = nsteps > 0;
  return check_launch(c, "rk_step");
}

int fst_rk_step_get_state(fst_ctx* c, int nsteps, double* U, size_t n) {
  if (!c || !U || nsteps < 0) return FST_ERR_INVALID;
  if (n != (size_t)c->g.sv * c->g.nvt) return fail(c, FST_ERR_SIZE, "state size mismatch");
  // (a copy into pageable memory returns only when it is done, which would
  // hold back the launches behind it: overlap into page-locked memory only)
  cudaPointerAttributes pa{};
  if (cudaPointerGetAttributes(&pa, U) != cudaSuccess) cudaGetLastError();
  const bool overlap = nsteps > 0 && c->cf.mode != FST_MODE_PLAIN_FP64 && c->g.ndim == 3 &&
                       !c->gen && pa.type == cudaMemoryTypeHost;
  if (!overlap) {
    const int rc = fst_rk_step(c, nsteps);
    return rc ? rc : fst_get_state(c, U, n);
  }
  if (!c->dl.side) {
    cudaError_t e = cudaStreamCreateWithFlags(&c->dl.side, cudaStreamNonBlocking);
    for (int q = 0; q < 3 && e == cudaSuccess; ++q)
      e = cudaEventCreateWithFlags(&c->dl.ev[q], cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(c, e, "download stream");
  }
  cudaEventRecord(c->ev0, c->stream);
  int rc = FST_OK;
  c->dl.host = U;
  c->dl.issued = 0;
  for (int s = 0; s < nsteps && !rc; ++s) {
    c->bm.dl = s + 1 == nsteps ? &c->dl : nullptr;  // the last step's stage 2 copies as it goes
    rc = one_step(c);
  }
  c->bm.dl = nullptr;
  if (rc) {
    cudaStreamSynchronize(c->dl.side);
    return rc;
  }
  cudaEventRecord(c->ev1, c->stream);
  c->timed = true;
  // groups no kernel completed on its own: after the whole stage
  const Geo& g = c->g;
  struct Grp {
    int bit, v0, nvar;
  } grps[3] = {{FST_DL_MOMENTA, 0, 4}, {FST_DL_SPECIES, 4, g.ns}, {FST_DL_CEQ, g.nv, g.nvt - g.nv}};
  cudaError_t e = cudaSuccess;
  for (const Grp& q : grps) {
    if ((c->dl.issued & q.bit) || q.nvar <= 0 || e != cudaSuccess) continue;
    const size_t off = (size_t)g.sv * q.v0;
    e = cudaMemcpyAsync(U + off, c->Ua + off, sizeof(double) * g.sv * q.nvar,
                        cudaMemcpyDeviceToHost, c->stream);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->dl.side);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "rk_step_get_state");
  return device_errors(c);
}

int fst_set_grid(fst_ctx* c, const double* nodes, size_t n) {
  if (!c || !nodes) return FST_ERR_INVALID;
  if (!c->gen) return fail(c, FST_ERR_UNSUPPORTED, "not a generalized-grid context");
  if (n != fst_grid_size(&c->cf)) return fail(c, FST_ERR_SIZE, "grid size mismatch");
  double* dX = nullptr;
  cudaError_t e = cudaMalloc(&dX, n * sizeof(double));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, FST_ERR_OOM, "grid buffer allocation failed");
  }
  const bool mixed = c->cf.mode != FST_MODE_PLAIN_FP64;
  double* met = mixed ? c->bm.met64 : c->g.ndim == 3 ? c->b3.met : c->b2.met;
  e = cudaMemcpyAsync(dX, nodes, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    c->stats.kernel_launches += fst_gen_metrics(c->g, dX, met, c->stream);
    if (mixed)
      c->stats.kernel_launches += fst_mixedgen_pair(c->g, c->bm.gq, met, c->bm.metf, c->stream);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(dX);
  if (e != cudaSuccess) return cuda_fail(c, e, "set_grid");
  c->grid_set = true;
  return FST_OK;
}

int fst_get_metrics(fst_ctx* c, double* out, size_t n) {
  if (!c || !out) return FST_ERR_INVALID;
  if (!c->gen) return fail(c, FST_ERR_UNSUPPORTED, "not a generalized-grid context");
  if (n != fst_metrics_size(&c->cf)) return fail(c, FST_ERR_SIZE, "metrics size mismatch");
  const double* met = c->cf.mode != FST_MODE_PLAIN_FP64 ? c->bm.met64
                     : c->g.ndim == 3                     ? c->b3.met
                                                          : c->b2.met;
  cudaError_t e = cudaMemcpyAsync(out, met, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "get_metrics");
  return FST_OK;
}

int fst_secondary(fst_ctx* c, double* out, size_t n) {
  if (!c || !out) return FST_ERR_INVALID;
  const Geo& g = c->g;
  const size_t nc = (size_t)g.sv;
  const int nf = g.ndim == 3 ? 6 : 5;
  if (n != nc * nf) return fail(c, FST_ERR_SIZE, "secondary size mismatch");
  const double *rho, *pr, *vel, *T;
  c->prof.begin("secondary", c->stream);
  if (c->cf.mode != FST_MODE_PLAIN_FP64) {
    c->stats.kernel_launches += fst_mixed_secondary(g, c->P, c->bm, c->Ua, c->stream, &rho, &pr, &vel, &T);
  } else if (g.ndim == 3) {
    c->stats.kernel_launches += fst_plain3d_secondary(g, c->P, c->b3, c->Ua, c->stream);
    rho = c->b3.rho; pr = c->b3.pr; vel = c->b3.vel; T = c->b3.T;
  } else {
    c->stats.kernel_launches += fst_plain2d_secondary(g, c->P, c->b2, c->Ua, c->stream);
    rho = c->b2.rho; pr = c->b2.pr; vel = c->b2.vel; T = c->b2.T;
  }
  c->prof.end(c->stream);
  int rc = check_launch(c, "secondary");
  if (rc) return rc;
  const size_t B = nc * sizeof(double);
  cudaError_t e = cudaSuccess;
  for (int d = 0; d < g.ndim && e == cudaSuccess; ++d)
    e = cudaMemcpyAsync(out + nc * d, vel + nc * d, B, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out + nc * g.ndim, pr, B, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out + nc * (g.ndim + 1), T, B, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out + nc * (g.ndim + 2), rho, B, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "secondary copy");
  return FST_OK;
}

int fst_status(fst_ctx* c, double* vmin, double* vmax, double* xmin, double* xmax) {
  if (!c || !vmin || !vmax) return FST_ERR_INVALID;
  if ((xmin == nullptr) != (xmax == nullptr)) return fail(c, FST_ERR_INVALID, "xmin/xmax");
  const Geo& g = c->g;
  const int nx = g.ndim + 3;
  StatusFields F{};
  int nf = g.nvt;
  for (int v = 0; v < g.nvt; ++v) F.f[v] = c->Ua + g.sv * v;
  if (xmin) {  // fresh secondaries, ordered as varx: velocity, p, T, rho
    const double *rho, *pr, *vel, *T;
    if (c->cf.mode != FST_MODE_PLAIN_FP64) {
      c->stats.kernel_launches +=
          fst_mixed_secondary(g, c->P, c->bm, c->Ua, c->stream, &rho, &pr, &vel, &T);
    } else if (g.ndim == 3) {
      c->stats.kernel_launches += fst_plain3d_secondary(g, c->P, c->b3, c->Ua, c->stream);
      rho = c->b3.rho; pr = c->b3.pr; vel = c->b3.vel; T = c->b3.T;
    } else {
      c->stats.kernel_launches += fst_plain2d_secondary(g, c->P, c->b2, c->Ua, c->stream);
      rho = c->b2.rho; pr = c->b2.pr; vel = c->b2.vel; T = c->b2.T;
    }
    for (int d = 0; d < g.ndim; ++d) F.f[nf++] = vel + g.sv * d;
    F.f[nf++] = pr;
    F.f[nf++] = T;
    F.f[nf++] = rho;
  }
  if (!c->dstat) {
    int rc = allocd(c, &c->dstat, 2 * (size_t)(FST_MAXV + 6));
    if (rc) return rc;
  }
  unsigned long long init[2 * (FST_MAXV + 6)];
  for (int q = 0; q < 2 * nf; ++q) init[q] = FST_KEY_LOWEST;
  cudaError_t e = cudaMemcpyAsync(c->dstat, init, sizeof(unsigned long long) * 2 * nf,
                                  cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "status init");
  c->prof.begin("status", c->stream);
  k_status<<<dim3(152, nf), 256, 0, c->stream>>>(g, F, c->dstat);
  c->prof.end(c->stream);
  c->stats.kernel_launches += 1;
  int rc = check_launch(c, "status");
  if (rc) return rc;
  unsigned long long h[2 * (FST_MAXV + 6)];
  e = cudaMemcpyAsync(h, c->dstat, sizeof(unsigned long long) * 2 * nf, cudaMemcpyDeviceToHost,
                      c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "status");
  for (int q = 0; q < nf; ++q) {
    const double mx = fst_unkey(h[2 * q]), mn = -fst_unkey(h[2 * q + 1]);
    if (q < g.nvt) {
      vmax[q] = mx;
      vmin[q] = mn;
    } else {
      xmax[q - g.nvt] = mx;
      xmin[q - g.nvt] = mn;
    }
  }
  (void)nx;
  return device_errors(c);
}

int fst_noise_filter(fst_ctx* c, const fst_noise_params* np) {
  if (!c || !np) return FST_ERR_INVALID;
  if (c->gen && c->g.ndim == 3)
    return fail(c, FST_ERR_UNSUPPORTED, "the generalized 3D module has no noise filter");
  if (np->nt < 0) return fail(c, FST_ERR_INVALID, "noise nt must be >= 0");
  c->bm.fused_for = nullptr;  // the filter changes the state's interior
  const Geo& g = c->g;
  if (!c->dnoise) {  // zero-initialised like the module's FS3D_I / FS2D_I
    const size_t ints = (size_t)fst_noise_ints(g);
    int rc = allocd(c, &c->dnoise, ints);
    if (!rc) rc = allocd(c, &c->dnoise_key, 1);
    if (rc) return rc;
    cudaError_t e = cudaMemsetAsync(c->dnoise, 0, sizeof(int) * ints, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "noise init");
  }
  c->stats.kernel_launches +=
      fst_noise_launch(g, c->cf, c->Ua, c->dnoise, c->dnoise_key, *np, c->stream, &c->prof,
                       &c->noise_graph);
  return check_launch(c, "noise filter");
}

int fst_fp64_rate(void* cuda_stream, double* gflops) {
  if (!gflops) return FST_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)cuda_stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, iters = 4096;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return FST_ERR_CUDA;
  k_fp64_rate<<<blocks, 256, 0, st>>>(nullptr, 64);  // warm-up
  cudaEventRecord(e0, st);
  k_fp64_rate<<<blocks, 256, 0, st>>>(nullptr, iters);
  cudaEventRecord(e1, st);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess || ms <= 0.f) return FST_ERR_CUDA;
  *gflops = 2.0 * 8.0 * iters * (double)blocks * 256.0 / (ms * 1e-3) / 1e9;
  return FST_OK;
}

int fst_check_finite(fst_ctx* c) {
  if (!c) return FST_ERR_INVALID;
  const long long n = c->g.sv * c->g.nvt;
  cudaMemsetAsync(c->dflag, 0, sizeof(int), c->stream);
  k_nonfinite<<<1216, 256, 0, c->stream>>>(c->Ua, n, c->dflag);
  c->stats.kernel_launches += 1;
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, c->dflag, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "check_finite");
  c->stats.nonfinite = h;
  if (h) return fail(c, FST_ERR_NONFINITE, "non-finite value in state");
  return device_errors(c);
}

int fst_get_stats(const fst_ctx* cc, fst_stats* out) {
  if (!cc || !out) return FST_ERR_INVALID;
  fst_ctx* c = const_cast<fst_ctx*>(cc);
  cudaStreamSynchronize(c->stream);
  *out = c->stats;
  const unsigned long long* red = c->cf.mode != FST_MODE_PLAIN_FP64 ? c->bm.red
                                  : c->g.ndim == 3 ? c->b3.red : c->b2.red;
  if (c->cf.ceq && red) {
    unsigned long long h[2] = {0, 0};
    if (cudaMemcpy(h, red, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess) {
      out->max_wave_speed = fst_unkey(h[0]);
      out->max_chat = fst_unkey(h[1]);
    }
  }
  if (c->timed) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) out->last_step_ms = ms;
  }
  out->flagged_face_fraction = fst_mixed_flagged_fraction(c->bm, c->stream);
  return FST_OK;
}

int fst_hybrid_features(fst_ctx* c, float* d_features, unsigned char* d_labels, size_t capacity,
                        float label_ratio, size_t* count) {
  if (!c || !d_features || !d_labels || !count) return FST_ERR_INVALID;
  if (c->cf.mode == FST_MODE_PLAIN_FP64) return fail(c, FST_ERR_UNSUPPORTED, "needs a mixed context");
  if (!c->bm.ymax) {  // mixed contexts get the hybrid work arrays on first use
    int rc = fst_hybrid_alloc(c->cf, c->g, c->bm, [&](void** p, size_t bytes) { return alloc(c, p, bytes); });
    if (rc) return rc;
  }
  if (c->g.ndim == 3) {
    int rc = bcs(c, c->Ua);
    if (rc) return rc;
  }
  c->bm.fused_for = nullptr;
  c->stats.kernel_launches += fst_mixed_prims(c->g, c->P, c->cf, c->bm, c->Ua, c->stream);
  const MixedView M{c->bm.Q, c->bm.rho32, c->bm.vel32, c->bm.p64,  c->bm.mu32, c->bm.nrg,
                    c->bm.C, c->bm.T32,   c->bm.rho64, c->bm.p32, c->bm.plo};
  int rc = fst_hybrid_features_impl(c->bm.gq, c->bm, M, d_features, d_labels, capacity,
                                    label_ratio, count, c->stream);
  if (rc) return fail(c, rc, "feature kernels");
  c->stats.kernel_launches += 2;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? FST_OK : cuda_fail(c, e, "features");
}

int fst_hybrid_set_params(fst_ctx* c, const float* params, float threshold) {
  if (!c || !params) return FST_ERR_INVALID;
  if (c->cf.mode != FST_MODE_HYBRID) return fail(c, FST_ERR_UNSUPPORTED, "needs a hybrid context");
  int rc = fst_hybrid_pack(c->bm, params, c->stream);
  if (rc) return fail(c, rc, "parameter upload");
  c->bm.threshold = threshold;
  c->bm.hyb_active = true;
  return FST_OK;
}

int fst_hybrid_get_counts(fst_ctx* c, fst_hybrid_counts* out, int reset) {
  if (!c || !out) return FST_ERR_INVALID;
  if (!c->bm.counters) return fail(c, FST_ERR_UNSUPPORTED, "needs a mixed context");
  unsigned long long h[8] = {0};
  cudaError_t e = cudaMemcpyAsync(h, c->bm.counters, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "counts");
  out->faces = (int64_t)h[0];
  out->weno_faces = (int64_t)h[1];
  out->audit_faces = (int64_t)h[2];
  out->audit_nonsmooth = (int64_t)h[3];
  out->audit_missed = (int64_t)h[4];
  if (reset) {
    e = cudaMemsetAsync(c->bm.counters, 0, sizeof(h), c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "counts reset");
  }
  return FST_OK;
}

int fst_set_profiling(fst_ctx* c, int on) {
  if (!c) return FST_ERR_INVALID;
  c->prof.on = on != 0;
  return FST_OK;
}

int fst_kernel_times(fst_ctx* c, fst_kernel_time* out, int max, int* count) {
  if (!c || (!out && max > 0)) return FST_ERR_INVALID;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "kernel_times sync");
  std::vector<fst_kernel_time> agg;
  for (auto& r : c->prof.recs) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    size_t q = 0;
    for (; q < agg.size(); ++q)
      if (std::strncmp(agg[q].name, r.name, sizeof(agg[q].name)) == 0) break;
    if (q == agg.size()) {
      fst_kernel_time t{};
      std::strncpy(t.name, r.name, sizeof(t.name) - 1);
      agg.push_back(t);
    }
    agg[q].launches += 1;
    agg[q].total_ms += ms;
    c->prof.pool.push_back(r.a);
    c->prof.pool.push_back(r.b);
  }
  c->prof.recs.clear();
  int n = 0;
  for (; n < (int)agg.size() && n < max; ++n) out[n] = agg[n];
  if (count) *count = n;
  return FST_OK;
}

}  // extern "C"
