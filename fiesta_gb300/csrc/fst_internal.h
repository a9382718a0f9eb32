// fst_internal.h — launch entry points shared between the libfst translation
// units (not part of the public ABI).
#pragma once
#include <cstddef>
#include <functional>

#include <string>
#include <vector>

#include "fst_common.cuh"

// Optional CUDA-event bracketing of kernel launches (fst_set_profiling).
struct Prof {
  bool on = false;
  struct Rec {
    const char* name;
    cudaEvent_t a, b;
  };
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t take() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  void begin(const char* name, cudaStream_t s) {
    if (!on) return;
    Rec r{name, take(), take()};
    cudaEventRecord(r.a, s);
    recs.push_back(r);
  }
  void end(cudaStream_t s) {
    if (!on || recs.empty()) return;
    cudaEventRecord(recs.back().b, s);
  }
  ~Prof() {
    for (auto& r : recs) {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// Launch with optional event bracketing; counts into `n`.
#define FST_LAUNCH(prof, name, st, n, ...) \
  do {                                      \
    if (prof) (prof)->begin(name, st);      \
    __VA_ARGS__;                            \
    if (prof) (prof)->end(st);              \
    ++(n);                                  \
  } while (0)

// fst_api.cu
std::string fst_setup_geo_phys(const fst_config* cfg, Geo& g, Phys& P);

// fst_gen.cu: metric tensor of a generalized grid from its node coordinates
int fst_gen_metrics(const Geo& g, const double* nodes, double* met, cudaStream_t st);

struct MixedView;
// fst_mixedgen.cu: the mixed path's generalized-grid pieces
int fst_mixedgen_pair(const Geo& g, const Geo& gq, const double* met, float* metf,
                      cudaStream_t st);
int fst_mixedgen_tvel(const Geo& g, const Geo& gq, const float* metf, float* vel,
                      cudaStream_t st);
int fst_mixedgen_cell(const Geo& g, const Geo& gq, const MixedView& M, const float* metf,
                      const double* Uold, double* Unew, double coef, double* Rout,
                      cudaStream_t st);

// fst_bc.cu
// n words of p set to v by a kernel on st (reduction-word resets)
void fst_fill_keys(unsigned long long* p, int n, unsigned long long v, cudaStream_t st);
int fst_launch_bcs(const Geo& g, const fst_config& cf, double* U, cudaStream_t stream, Prof* prof);

// fst_plain3d.cu
struct Plain3DBufs {
  double *rho, *pr, *vel, *Y, *nrg, *T;
  double *F, *S, *MF;
  unsigned long long* red;
  double* met;  // generalized grids: metric tensor (ngi,ngj,ngk,3,3), else null
};
int fst_plain3d_stage(const Geo& g, const Phys& P, const Plain3DBufs& b, const double* Uin,
                      const double* Uold, double* Unew, double coef, double* Rout, bool ghosts,
                      cudaStream_t st, Prof* prof);
int fst_plain3d_secondary(const Geo& g, const Phys& P, const Plain3DBufs& b, const double* U,
                          cudaStream_t st);

// fst_plain2d.cu
struct Plain2DBufs {
  double *rho, *pr, *vel, *T, *nrg;
  double *F, *S, *Q, *MF;
  double* met;  // generalized grids: metric tensor (ngi,ngj,2,2), else null
  unsigned long long* red;
};
int fst_plain2d_stage(const Geo& g, const Phys& P, const Plain2DBufs& b, const double* Uin,
                      const double* Uold, double* Unew, double coef, double* Rout, bool ghosts,
                      cudaStream_t st, Prof* prof);
int fst_plain2d_secondary(const Geo& g, const Phys& P, const Plain2DBufs& b, const double* U,
                          cudaStream_t st);

// fst_mixed.cu (FST_MODE_MIXED / FST_MODE_HYBRID)
struct Mixed3DMaps;  // TMA tensor maps of the 3D primitive arrays (fst_mixed3d.cu)
// The second set of 3D primitive arrays, the tensor maps over them and its
// reduction words (see MixedBufs::fused)
struct PrimSet {
  float *Q, *rho32, *vel32, *mu32, *nrg, *C, *p32, *plo;
  double* rho64;
  Mixed3DMaps* maps3d;
  unsigned long long* red;
};
// fst_rk_step_get_state: during the final stage, each variable group of
// U_new is copied to `host` on stream `side` as soon as the last kernel that
// writes it has run (bits of `issued`: 1 the C variables, 2 the species,
// 4 the momenta and energy)
struct MixedDownload {
  double* host;
  cudaStream_t side;
  cudaEvent_t ev[3];
  int issued;
};
constexpr int FST_DL_CEQ = 1, FST_DL_SPECIES = 2, FST_DL_MOMENTA = 4;
struct MixedBufs {
  // Geometry of the primitive arrays.  2D: the state's.  3D: rows padded to
  // a multiple of 4 floats so that every row, plane and field starts on a
  // 16-byte boundary, as TMA tensor maps require.
  Geo gq;
  // FP32 primitives written by the mixed primitive pass; mu32 is the
  // mixture viscosity sum_s Y_s mu_s of a cell (3D viscous runs)
  float *Q, *rho32, *vel32, *mu32, *T32, *nrg, *C;
  double* p64;    // FP64 pressure (2D)
  float* p32;     // pressure as an FP32 pair: hi [cells], lo [cells] (3D)
  double* rho64;  // FP64 density (buoyancy source)
  // 3D C-equation runs: low parts of the FP32 pairs of rho, nrg, u, v, w
  // ([5][cells], see Prim3Out) for the shock/contact switches
  float* plo;
  // FP64 secondary outputs (fst_secondary)
  double *rho, *pr, *vel, *T;
  unsigned long long* red;
  unsigned long long* counters;  // hybrid: [0] faces classified, [1] routed to WENO
  // hybrid smoothness classifier
  bool hyb_active;
  unsigned char* smooth;   // [cells][3] 1 = linear upwind on that face
  float* ymax;             // largest mass fraction per cell
  void* mlp;               // device weights (fst_hybrid.cu)
  float threshold, label_ratio;
  int audit_every;
  int classify_every;
  // step bookkeeping (set by fst_rk_step): classify at stage 1 (or for a
  // bare RHS), reuse at stage 2; audit steps run full WENO
  long long step;
  int stage;
  bool classified;
  // 3D fused kernels: tensor maps (host copy, passed by value at launch)
  // and the device error word (FST_DEVERR_* bits; a TMA wait that ran out)
  Mixed3DMaps* maps3d;
  unsigned int* dev_err;
  // generalized 3D grids: the FP64 metric tensor (state layout, 9 fields)
  // and its FP32 pairs hi [9] + lo [9] in the primitives' layout
  double* met64;
  float* metf;
  // Fused 3D stages (cartesian, up to 5 species): the last kernel of a stage
  // writes the primitives of U_new's interior into `alt`, which becomes the
  // current set for the next stage; its ghost cells are filled after the
  // boundary conditions.  fused_for: the state whose interior primitives the
  // current set holds (null when none does, e.g. after the state was set).
  bool fused;
  PrimSet alt;
  const double* fused_for;
  // set by fst_rk_step_get_state for the final stage only
  MixedDownload* dl;
};
// exchange the current primitive set with b.alt
void fst_mixed_swap(MixedBufs& b);
struct MixedView {
  const float* Q;    // [nv][cells] conserved variables, Q[ndim] = E + p
  const float* rho;  // [cells]
  const float* vel;  // [ndim][cells]
  const double* p;   // [cells] FP64 pressure (2D)
  const float* mu;   // [cells] mixture viscosity (3D viscous)
  const float* nrg;  // [cells]
  const float* C;    // [5][cells]
  const float* T;    // [cells] (2D viscous heat flux)
  const double* rho64;  // [cells] FP64 density (buoyancy)
  const float* pp;      // [2][cells] pressure hi + lo (3D)
  const float* lo;      // [5][cells] low parts of rho, nrg, u, v, w (3D C-equation)
};
using fst_alloc_fn = std::function<int(void**, size_t)>;
size_t fst_mixed_work_doubles_per_cell(const fst_config& cf, const Geo& g);
// Fill the primitive arrays with NaN bytes (debug canary, FST_DEBUG_CANARY)
cudaError_t fst_mixed_canary(const Geo& g, const MixedBufs& b, cudaStream_t st);
int fst_mixed_alloc(const fst_config& cf, const Geo& g, MixedBufs& b, const fst_alloc_fn& alloc,
                    std::string* why);
int fst_mixed_stage(const Geo& g, const Phys& P, const fst_config& cf, MixedBufs& b,
                    const double* Uin, const double* Uold, double* Unew, double coef, double* Rout,
                    bool ghosts, cudaStream_t st, Prof* prof);
int fst_mixed_secondary(const Geo& g, const Phys& P, const MixedBufs& b, const double* U,
                        cudaStream_t st, const double** rho, const double** pr, const double** vel,
                        const double** T);
double fst_mixed_flagged_fraction(const MixedBufs& b, cudaStream_t st);

// fst_hybrid.cu (FST_MODE_HYBRID)
int fst_hybrid_alloc(const fst_config& cf, const Geo& g, MixedBufs& b, const fst_alloc_fn& alloc);
int fst_hybrid_classify(const Geo& g, const Phys& P, const MixedBufs& b, const MixedView& M,
                        cudaStream_t st, Prof* prof, const unsigned char** smooth, bool audit);
int fst_hybrid_features_impl(const Geo& g, const MixedBufs& b, const MixedView& M, float* out,
                             unsigned char* lab, size_t cap, float ratio, size_t* count,
                             cudaStream_t st);
int fst_hybrid_pack(MixedBufs& b, const float* h_params, cudaStream_t st);
int fst_mixed_prims(const Geo& g, const Phys& P, const fst_config& cf, const MixedBufs& b,
                    const double* U, cudaStream_t st);
// Fused upload (3D fused stages): copy the state from host memory the GPU can
// read (Uh, a device-visible pointer to pinned memory) into U while computing
// the primitives of its interior and the C-equation maxima, as the previous
// stage's epilogue would have; the first stage then fills only the ghost
// cells.  Returns the kernel launches, or -1 when the context's stages are
// not fused (the caller copies instead).
int fst_mixed_upload(const Geo& g, const Phys& P, MixedBufs& b, const double* Uh, double* U,
                     cudaStream_t st, Prof* prof);

// fst_noise.cu: the postStep noise filter on state U; `noise` holds
// fst_noise_ints(g) ints (the indicator, then the removal's tile marks).
// The tile marks and removal sweeps (about a hundred short launches) run as
// a CUDA graph, captured on a private stream at the first unprofiled call
// and replayed while their launch parameters stay the same.
struct NoiseGraph {
  cudaStream_t cap = nullptr;  // capture stream (the caller's may be the legacy stream)
  cudaGraphExec_t exec = nullptr;
  unsigned char sig[128] = {};
  int launches = 0;
};
void fst_noise_graph_release(NoiseGraph& ng);
long long fst_noise_ints(const Geo& g);
int fst_noise_launch(const Geo& g, const fst_config& cf, double* U, int* noise,
                     unsigned long long* key, const fst_noise_params& np, cudaStream_t st,
                     Prof* prof, NoiseGraph* graph);

// fst_mixed3d.cu: the 3D mixed/hybrid right-hand side + RK stage (two
// fused kernels fed by TMA plane loads) and its tensor maps
Geo fst_prim_geo(const Geo& g);
int fst_mixed3d_prepare(const Geo& g, MixedBufs& b, std::string* why);
void fst_mixed3d_release(MixedBufs& b);
// fused: the stage also writes the primitives of U_new's interior into b.alt
int fst_mixed3d_rhs(const Geo& g, const Phys& P, const MixedBufs& b, const MixedView& M,
                    const unsigned char* smooth, const double* Uold, double* Unew, double coef,
                    double* Rout, cudaStream_t st, Prof* prof, bool hybrid, bool fused);
