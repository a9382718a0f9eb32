// fst_noalloc.cu — fst_rhs2d_noalloc: the plain FP64 2D right-hand side with
// its work arrays in one fixed device array instead of cudaMalloc'd memory,
// for host programs that manage all device memory themselves and cannot let
// a library allocate (see include/fst.h).
//
// Scratch: g_scratch below, FST_NOALLOC_SCRATCH_BYTES of device memory that
// every GPU loading the library holds until the process exits.  In host code
// `g_scratch` is only a host-side stand-in for that symbol, not a device
// address; each device's address is looked up once with cudaGetSymbolAddress
// while that device is current, on the first call made on it.
#include <cstdio>
#include <mutex>

#include "fst_internal.h"

namespace {

constexpr size_t kScratchDoubles = FST_NOALLOC_SCRATCH_BYTES / sizeof(double);
static __device__ __align__(256) double g_scratch[kScratchDoubles];

// Work doubles per cell: rho, p, u, v, T, e (6), the face fluxes (2 nv),
// with viscosity the stress (6) and heat flux (2), with the C-equation the
// face tensors (8); plus two reduction words per call.
constexpr size_t work_per_cell(int nv, bool visc, bool ceq) {
  return 6 + 2 * (size_t)nv + (visc ? 8 : 0) + (ceq ? 8 : 0);
}
// The largest 2D mixture (nv = 3 + FST_MAX_SPECIES, viscous, C-equation) on
// the largest accepted grid fits the array, so the cell count is the only
// limit a caller meets.
static_assert((size_t)FST_NOALLOC_MAX_CELLS * work_per_cell(3 + FST_MAX_SPECIES, true, true) + 2 <=
                  kScratchDoubles,
              "the fixed scratch array must hold the largest accepted 2D grid");

constexpr int kMaxDevices = 64;
std::mutex g_lock;
double* g_addr[kMaxDevices] = {nullptr};

// Device address of g_scratch on the current device (set up on first use).
int scratch_address(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "fst_rhs2d_noalloc: cudaGetDevice: %s\n", cudaGetErrorString(e));
    return FST_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    std::fprintf(stderr, "fst_rhs2d_noalloc: device index %d is beyond the %d supported\n", dev,
                 kMaxDevices);
    return FST_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> guard(g_lock);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
      std::fprintf(stderr, "fst_rhs2d_noalloc: cudaGetSymbolAddress: %s\n", cudaGetErrorString(e));
      return FST_ERR_CUDA;
    }
    g_addr[dev] = (double*)p;
  }
  *out = g_addr[dev];
  return FST_OK;
}

}  // namespace

extern "C" int fst_rhs2d_noalloc(const fst_config* cfg, const double* d_U, double* d_R, size_t n,
                                 void* cuda_stream) {
  if (!cfg || !d_U || !d_R) return FST_ERR_INVALID;
  // An error left pending by the caller's own earlier work is reported as
  // such and left in place, so that a launch failure below is ours alone.
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    std::fprintf(stderr, "fst_rhs2d_noalloc: a CUDA error from earlier work is pending: %s\n",
                 cudaGetErrorString(e));
    return FST_ERR_CUDA;
  }
  Geo g;
  Phys P;
  const std::string why = fst_setup_geo_phys(cfg, g, P);
  if (!why.empty()) {
    std::fprintf(stderr, "fst_rhs2d_noalloc: %s\n", why.c_str());
    return FST_ERR_INVALID;
  }
  if (g.ndim != 2 || cfg->mode != FST_MODE_PLAIN_FP64 || cfg->grid_type != FST_GRID_CARTESIAN) {
    std::fprintf(stderr, "fst_rhs2d_noalloc: needs a 2D cartesian plain FP64 config\n");
    return FST_ERR_UNSUPPORTED;
  }
  const size_t cells = (size_t)g.sv;
  if (n != cells * (size_t)g.nvt) return FST_ERR_SIZE;
  const size_t need = cells * work_per_cell(g.nv, cfg->visc != 0, cfg->ceq != 0) + 2;
  if (cells > FST_NOALLOC_MAX_CELLS || need > kScratchDoubles) {
    std::fprintf(stderr,
                 "fst_rhs2d_noalloc: grid of %zu cells (with ghosts) needs %zu work doubles; "
                 "the limits are %d cells and %zu doubles\n",
                 cells, need, FST_NOALLOC_MAX_CELLS, kScratchDoubles);
    return FST_ERR_SIZE;
  }
  double* base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)cuda_stream;

  Plain2DBufs b{};
  double* q = base;
  auto take = [&](size_t count) {
    double* p = q;
    q += count;
    return p;
  };
  b.red = (unsigned long long*)take(2);
  b.rho = take(cells);
  b.pr = take(cells);
  b.vel = take(2 * cells);
  b.T = take(cells);
  b.nrg = take(cells);
  b.F = take(2 * (size_t)g.nv * cells);
  if (cfg->visc) {
    b.S = take(6 * cells);
    b.Q = take(2 * cells);
  }
  if (cfg->ceq) b.MF = take(8 * cells);

  // the right-hand side is zero outside the interior, like the reference's
  // zero-initialised dvar; the interior is overwritten below
  e = cudaMemsetAsync(d_R, 0, n * sizeof(double), st);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "fst_rhs2d_noalloc: cudaMemsetAsync: %s\n", cudaGetErrorString(e));
    return FST_ERR_CUDA;
  }
  fst_plain2d_stage(g, P, b, d_U, nullptr, nullptr, 0.0, d_R, false, st, nullptr);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    std::fprintf(stderr, "fst_rhs2d_noalloc: launch: %s\n", cudaGetErrorString(e));
    return FST_ERR_CUDA;
  }
  return FST_OK;
}
