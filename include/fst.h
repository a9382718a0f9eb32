/*
 * fst.h — C ABI of libfst, the GB300 (sm_103a) implementation of FIESTA's
 * per-Runge-Kutta-stage right-hand side and update: uniform Cartesian grids
 * (the cart2d / cart3d modules) and generalized curvilinear grids (the
 * gen2d / gen3d modules).
 *
 * Everything crossing this boundary is plain C: a config struct, pointers and
 * sizes.  No C++, Kokkos or torch types appear in any signature.
 *
 * State layout (host and device buffers alike): the layout FIESTA's CUDA build
 * gives `FS4D var(ngi, ngj, ngk, nvt)` (Kokkos LayoutLeft, i fastest):
 *
 *     U[i + ngi*(j + ngj*(k + ngk*v))]     ngi = nci + 2*ng, ngk = 1 in 2D
 *
 * with ng = 3 ghost layers.  Variable order follows the reference:
 *   3D: x-, y-, z-momentum, total energy, ns species densities, then (ceq) the
 *       five C-equation variables C, C_hat, C_1, C_2, C_3
 *       (src/cart3d.cpp:98-110 of the reference);
 *   2D: x-, y-momentum, energy, ns species densities, then (ceq) C, C_hat,
 *       Tau_1, Tau_2, Debug (src/cart2d.cpp:40-58).
 *
 * Every function returns FST_OK (0) or a negative status; fst_last_error()
 * gives the message.  The reference calls exit(EXIT_FAILURE) instead
 * (src/bc.cpp:266-268, src/luaReader.cpp:100-101).
 *
 * Threading: one context per host thread; all work is ordered on the
 * context's CUDA stream.  There is no global mutable state.
 */
#ifndef FST_H
#define FST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FST_ABI_VERSION 1
#define FST_MAX_SPECIES 16

/* Status codes. */
enum {
  FST_OK = 0,
  FST_ERR_INVALID = -1,     /* bad argument or config                        */
  FST_ERR_OOM = -2,         /* device or host allocation failed / size limit */
  FST_ERR_CUDA = -3,        /* a CUDA runtime call failed                    */
  FST_ERR_TIMEOUT = -4,     /* a bounded device-side wait gave up            */
  FST_ERR_NONFINITE = -5,   /* a NaN/Inf was found in the state              */
  FST_ERR_UNSUPPORTED = -6, /* valid FIESTA option this path does not cover  */
  FST_ERR_SIZE = -7         /* caller buffer size does not match the grid    */
};

/* Boundary condition types; values match the order of the reference's
 * `enum class BCType {outflow, reflective, noslip, hydrostatic}`
 * (src/bc.hpp:31). */
enum {
  FST_BC_OUTFLOW = 0,
  FST_BC_REFLECTIVE = 1,
  FST_BC_NOSLIP = 2,
  FST_BC_HYDROSTATIC = 3
};

/* Arithmetic of the right-hand side. */
enum {
  FST_MODE_PLAIN_FP64 = 0, /* the reference's FP64 arithmetic, operation for
                              operation (bitwise reproducible)              */
  FST_MODE_MIXED = 1,      /* FP32 reconstruction / fluxes / viscous / C-eq;
                              FP64 state, EOS recovery and RK combine       */
  FST_MODE_HYBRID = 2      /* MIXED + learned smoothness classifier routing
                              smooth faces to the linear upwind flux        */
};

/* Grid type (fiesta.grid.type, src/input.cpp:287-350).  GENERALIZED runs the
 * reference's gen2d / gen3d modules (src/gen2d.cpp, src/gen3d.cpp): curvilinear
 * node coordinates given by fst_set_grid, metric terms on every cell; plain
 * FP64 (2D and 3D) or, in 3D, FST_MODE_MIXED. */
enum {
  FST_GRID_CARTESIAN = 0,
  FST_GRID_GENERALIZED = 1
};

/* 2D advection scheme (fiesta.advection_scheme, src/input.cpp:317-323); the
 * 3D modules always use WENO5.  0 means WENO5. */
enum {
  FST_SCHEME_WENO5 = 1,
  FST_SCHEME_CENTERED4 = 2, /* computeFluxCentered2D (src/flux.hpp:108-167) */
  FST_SCHEME_QUICK = 3      /* computeFluxQuick2D (src/flux.hpp:169-221)    */
};

/*
 * Run configuration: the fields of the reference's `struct inputConfig`
 * (src/input.hpp:59-148) that the RHS path reads, filled from the same Lua
 * deck keys (src/input.cpp:139-308).
 */
typedef struct fst_config {
  int abi_version;           /* must be FST_ABI_VERSION                     */
  int ndim;                  /* 2 or 3 (fiesta.grid.ndim)                   */
  int nci, ncj, nck;         /* interior cells (fiesta.grid.ni); nck=1 in 2D */
  int ng;                    /* ghost layers; must be 3 (fiesta.ng)         */
  double dx, dy, dz;         /* cell sizes (fiesta.grid.dx); 2D: dz ignored */
  double dt;                 /* fixed time step (fiesta.time.dt)            */
  int ns;                    /* number of species (#fiesta.species)         */
  double R;                  /* universal gas constant (fiesta.R)           */
  double gamma[FST_MAX_SPECIES]; /* species ratio of specific heats         */
  double M[FST_MAX_SPECIES];     /* species molar mass                      */
  double mu[FST_MAX_SPECIES];    /* species dynamic viscosity               */
  int visc;                  /* fiesta.viscosity.enabled                    */
  int ceq;                   /* fiesta.ceq.enabled                          */
  double kap, eps, alpha;    /* fiesta.ceq.kappa / epsilon / alpha          */
  int buoyancy;              /* fiesta.buoyancy.enabled                     */
  double g_accel, rho_ref;   /* fiesta.buoyancy.acceleration / rho_reference */
  int xper, yper, zper;      /* fiesta.bc.{x,y,z}periodic                   */
  int bc_xmin, bc_xmax, bc_ymin, bc_ymax, bc_zmin, bc_zmax; /* FST_BC_*     */
  int mode;                  /* FST_MODE_*                                  */
  int audit_every;           /* HYBRID: full-WENO audit step period (0: never) */
  int classify_every;        /* HYBRID: steps between classifications (0, 1: every step) */
  int grid_type;             /* FST_GRID_* (fiesta.grid.type)               */
  int scheme;                /* FST_SCHEME_* (fiesta.advection_scheme), 0 = WENO5 */
  int reserved[5];           /* zero                                        */
} fst_config;

/* Per-context statistics (fst_stats). */
typedef struct fst_stats {
  double max_wave_speed;     /* maxS of the last C-equation stage           */
  double max_chat;           /* maxCh of the last C-equation stage          */
  double last_step_ms;       /* device time of the last fst_rk_step call    */
  double flagged_face_fraction; /* HYBRID: WENO share of faces, last stage  */
  int64_t steps;             /* RK steps taken since creation               */
  int64_t kernel_launches;   /* kernels launched since creation             */
  int nonfinite;             /* 1 if the last check found NaN/Inf           */
  int reserved[7];
} fst_stats;

typedef struct fst_ctx fst_ctx;

/* Fill `cfg` with defaults (the reference's deck defaults where it has them:
 * R = 8.314462, ng = 3, outflow BCs, plain FP64). */
void fst_config_defaults(fst_config* cfg);

/* Size of one state array in doubles: ngi*ngj*ngk*nvt. */
size_t fst_state_size(const fst_config* cfg);

/* Number of total variables nvt (nv + 5 with the C-equation). */
int fst_nvt(const fst_config* cfg);

/* Replaces the reference's cart3d_func / cart2d_func constructors
 * (src/cart3d.cpp:44-174, src/cart2d.cpp:29-134): validates the config,
 * allocates the device state and work arrays, uploads the species table.
 * The state starts at zero like a fresh Kokkos View. */
int fst_create(const fst_config* cfg, fst_ctx** out);
void fst_destroy(fst_ctx* ctx);
const char* fst_last_error(const fst_ctx* ctx);

/* Optional: order all work on this cudaStream_t (default: a private stream). */
int fst_set_stream(fst_ctx* ctx, void* cuda_stream);
int fst_synchronize(fst_ctx* ctx);

/* State transfer from / to host memory, LayoutLeft, n = fst_state_size().
 * Replaces the deep_copy of loadInitialConditions (src/input.cpp:515) and
 * the restart reader / writer's state access. */
int fst_set_state(fst_ctx* ctx, const double* U, size_t n);
int fst_get_state(fst_ctx* ctx, double* U, size_t n);
/* (3D mixed / hybrid contexts on cartesian grids with up to 5 species,
 * U in page-locked memory the GPU can read, i.e. cudaHostAlloc'd or
 * registered, on a device with pageable memory access such as a Grace
 * system: fst_set_state reads U with a kernel that also computes the
 * interior primitives on the way, so the next step skips that pass.  The
 * result is bit for bit that of the copy; FST_NO_FUSED_UPLOAD=1 in the
 * environment selects the copy.) */

/* `nsteps` time steps (as fst_rk_step) and the resulting state copied to host
 * memory U, as fst_get_state.  On 3D mixed / hybrid cartesian contexts the
 * copy of each variable group starts during the last stage, as soon as the
 * kernel that completes it has run (the C variables after the C-equation
 * kernel, then the momenta and energy, then the species), so the copy
 * overlaps the end of the step; elsewhere it follows the step.  Returns after
 * the copy. */
int fst_rk_step_get_state(fst_ctx* ctx, int nsteps, double* U, size_t n);

/* Same, from / to device memory on the context's GPU (no host staging). */
int fst_set_state_device(fst_ctx* ctx, const double* d_U, size_t n);
int fst_get_state_device(fst_ctx* ctx, double* d_U, size_t n);

/* Ghost fill of the current state: replaces applyBCs (src/bc.cpp:179-249)
 * with periodic self-copies in the order x, y, z (src/bc.cpp:202-214) and
 * then the face fills x-, x+, y-, y+, z-, z+ (src/bc.cpp:217-247). */
int fst_apply_bcs(fst_ctx* ctx);

/* One right-hand-side evaluation of the current state: replaces
 * cart3d_func::compute (src/cart3d.cpp:220-298, which applies BCs first),
 * cart2d_func::compute (src/cart2d.cpp:151-237, which does not), and on
 * generalized grids gen3d_func::compute / gen2d_func::compute
 * (src/gen3d.cpp:338-370, src/gen2d.cpp:103-130: no BCs, no viscous, buoyancy
 * or C-equation terms).  If R is not NULL the RHS `dvar` (LayoutLeft, zero
 * outside the interior) is copied to it.  n = fst_state_size(). */
int fst_compute_rhs(fst_ctx* ctx, double* R, size_t n);

/* `nsteps` time steps: each is preStep (cartesian 2D: applyBCs,
 * src/cart2d.cpp:147-149; nothing on generalized grids) followed by
 * rkAdvance (src/rk.cpp:28-70): two RHS evaluations and the two stage
 * combines. */
int fst_rk_step(fst_ctx* ctx, int nsteps);

/* Secondary variables of the current state over all cells, replacing
 * calculateRhoPT + computeVelocity + copyExtraVars (src/secondary.hpp:25-151):
 * 3D: u, v, w, p, T, rho (6 fields); 2D: u, v, p, T, rho (5 fields), each
 * LayoutLeft (ngi, ngj, ngk, nfields).  n = ngi*ngj*ngk*nfields. */
int fst_secondary(fst_ctx* ctx, double* varx, size_t n);

/* Scan the state for NaN/Inf (sets stats.nonfinite); FST_ERR_NONFINITE if any. */
int fst_check_finite(fst_ctx* ctx);

/* FP64 fused multiply-add throughput of the current device, in GFLOP/s
 * (2 per FMA), timed on `cuda_stream` with a kernel of independent FMA
 * chains over every SM.  No counterpart in the reference: it is the FP64
 * roof against which the plain FP64 path's kernels are judged. */
int fst_fp64_rate(void* cuda_stream, double* gflops);

/* Interior minimum and maximum of every state variable (vmin/vmax: nvt
 * values) and, when xmin/xmax are given, of the secondary variables of
 * fst_secondary recomputed from the current state (ndim+3 values: velocity,
 * p, T, rho) -- the reductions of statusCheck (src/status.cpp:116-253),
 * computed on the device.  As there, NaN is skipped and a variable without
 * a value above -DBL_MAX (below +DBL_MAX) reports that identity. */
int fst_status(fst_ctx* ctx, double* vmin, double* vmax, double* xmin, double* xmax);

int fst_get_stats(const fst_ctx* ctx, fst_stats* out);

/* Noise filter parameters: fiesta.noise.{dh, eta, coff, nt, mode}
 * (src/input.cpp:270-277). */
typedef struct fst_noise_params {
  double dh;                 /* detection threshold factor                   */
  double eta;                /* diffusion coefficient of the removal sweep   */
  double coff;               /* C_hat cutoff factor (used when ceq is on)    */
  int nt;                    /* removal sweeps per variable                  */
  int mode;                  /* 1: momenta; otherwise the energy             */
  int reserved[6];
} fst_noise_params;

/* The postStep noise filter of the current state (src/cart3d.cpp:319-374,
 * src/cart2d.cpp:257-307; detectNoise / removeNoise, src/noise.hpp:26-262):
 * per filtered variable, detection on a lattice of 3x3(x3) blocks, then `nt`
 * in-place diffusion sweeps over the flagged cells.  The reference's removal
 * updates the state in place while neighbours read it, so its result is that
 * of a sweep in loop order (i slowest); this entry point reproduces that
 * order exactly (tile wavefronts), giving the reference's serial result bit
 * for bit.  The noise indicator persists between calls, as the module's
 * member array does.  On a generalized 2D grid it is gen2d_func's variant
 * (src/gen2d.cpp:150-179: lattice from nci - 1, no cutoff, both momenta);
 * the generalized 3D module has none (FST_ERR_UNSUPPORTED).  The first call
 * with profiling off captures the removal sweeps into a CUDA graph on a
 * private stream (make it outside any stream capture of the caller); later
 * calls with the same parameters replay it. */
int fst_noise_filter(fst_ctx* ctx, const fst_noise_params* np);

/* Node coordinates of a generalized grid: (ni, nj, nk, 3) doubles, LayoutLeft,
 * ni = nci + 1, nj = ncj + 1, nk = nck + 1 in 3D and 1 in 2D (the reference's
 * `grid` view, src/gen3d.cpp:41, src/gen2d.cpp:25; filled by loadGrid,
 * src/input.cpp:529-560).  The 2D third component is ignored. */
size_t fst_grid_size(const fst_config* cfg);

/* Load the node coordinates and compute the metric tensor on every cell:
 * replaces loadGrid + gen3d_func::preSim / gen2d_func::preSim
 * (src/gen3d.cpp:129-335, src/gen2d.cpp:190-320): computeMetrics3D/2D
 * (src/metric.hpp:22-166) on the interior, then the ghost layers mirrored
 * from the interior in the reference's order.  Required before the first
 * right-hand side of an FST_GRID_GENERALIZED context. */
int fst_set_grid(fst_ctx* ctx, const double* nodes, size_t n);

/* The metric tensor of a generalized context, LayoutLeft:
 * 3D (ngi, ngj, ngk, 3, 3), 2D (ngi, ngj, 2, 2) — the reference's `metrics`
 * view.  n = fst_metrics_size(). */
size_t fst_metrics_size(const fst_config* cfg);
int fst_get_metrics(fst_ctx* ctx, double* out, size_t n);

/* Per-kernel device timing (the reference's per-region fiestaTimer,
 * src/timer.hpp:52-119, reset/accumulated around kernels in
 * src/cart3d.cpp:201-218).  With profiling on, every kernel launch is
 * bracketed by CUDA events on the context's stream; fst_kernel_times
 * synchronises, sums the times per kernel name since the last call, and
 * clears them.  `count` receives the number of entries written (<= max). */
typedef struct fst_kernel_time {
  char name[48];
  int64_t launches;
  double total_ms;
} fst_kernel_time;
int fst_set_profiling(fst_ctx* ctx, int on);
int fst_kernel_times(fst_ctx* ctx, fst_kernel_time* out, int max, int* count);

/* Allocation-free 2D right-hand side.  No counterpart in the reference: it
 * serves host programs that own every byte of device memory themselves (a
 * fixed pre-reserved pool, a Fortran or legacy host that forbids allocation
 * after start-up, a loop that cannot afford the implicit device-wide
 * synchronisation of cudaMalloc/cudaFree) and so cannot create an fst_ctx.
 *
 * Computes the plain FP64 right-hand side of cart2d_func::compute for the
 * device state d_U (LayoutLeft, ghosts already filled, n = fst_state_size())
 * into device memory d_R (same layout; zero outside the interior), on
 * `cuda_stream` (NULL: the default stream).  cfg must be 2D plain FP64.
 * Work arrays live in one fixed device array of FST_NOALLOC_SCRATCH_BYTES
 * inside the library (held by every GPU that loads it until exit).  A call
 * needs cells * (6 + 2 nv + 8 visc + 8 ceq) + 2 doubles of it (cells =
 * ngi*ngj including ghosts, nv = 3 + ns); the array holds that for every
 * mixture up to FST_MAX_SPECIES, so the limit a caller meets is
 * FST_NOALLOC_MAX_CELLS cells: larger grids return FST_ERR_SIZE.  Nothing is
 * allocated or freed.  Other configs (3D, mixed or hybrid mode, generalized
 * grids) return FST_ERR_UNSUPPORTED; null pointers FST_ERR_INVALID; a CUDA
 * error already pending from the caller's earlier work FST_ERR_CUDA, without
 * clearing it.  Devices with an index of 64 or more are not supported.
 * The first call on each device looks up that device's copy of the array
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the array: calls that overlap on the GPU (different
 * streams or host threads without ordering between them) race. */
#define FST_NOALLOC_MAX_CELLS 16384
#define FST_NOALLOC_SCRATCH_BYTES (8u << 20)
int fst_rhs2d_noalloc(const fst_config* cfg, const double* d_U, double* d_R, size_t n,
                      void* cuda_stream);

/* Batched 2D ensemble: many independent 2D cases of uneven size advanced
 * together in FST_MODE_MIXED.  Replaces running one cart2d_func per case
 * (src/main.cpp:40-72 once per deck).  Every case must be 2D, mixed, and
 * share ns and the visc / ceq / buoyancy switches; grids, spacings, time
 * steps, gases, gravity and BCs may differ.  Per RK stage the whole ensemble
 * takes one persistent launch of the fused RHS over a (case, tile) work list;
 * a time step (preStep BCs + two stages) is one CUDA graph replay. */
typedef struct fst_batch fst_batch;
typedef struct fst_batch_info_t {
  int ncases;
  int tile_height;        /* threads along j of the RHS tile (4, 8 or 16)  */
  int tiles;              /* work items per stage                         */
  int persistent_blocks;  /* blocks of the persistent RHS launch          */
  int launches_per_step;  /* kernels in the captured step graph           */
  int tile_width;         /* threads along i of the RHS tile (16, 32, 64) */
  int64_t interior_cells; /* sum over cases                               */
  int blocks_per_sm;      /* persistent blocks per SM in use              */
  int max_blocks_per_sm;  /* the occupancy limit of the tile shape        */
  int tune_candidates;    /* candidates the autotuner timed (0: not tuned) */
  int reserved;
  double tune_best_ms;    /* ms per step of the chosen candidate          */
  double tune_worst_ms;   /* ms per step of the slowest candidate         */
} fst_batch_info_t;
int fst_batch_create(const fst_config* cfgs, int ncases, fst_batch** out);
void fst_batch_destroy(fst_batch* b);
const char* fst_batch_last_error(const fst_batch* b);
int fst_batch_set_state(fst_batch* b, int case_index, const double* U, size_t n);
int fst_batch_get_state(fst_batch* b, int case_index, double* U, size_t n);
int fst_batch_rk_step(fst_batch* b, int nsteps);
int fst_batch_synchronize(fst_batch* b);
void* fst_batch_stream(fst_batch* b);  /* the cudaStream_t the graph runs on */
/* RHS tile shape: width x height threads, (16|32) x (4|8|16) or 64 x (4|8),
 * and persistent blocks per SM (0: the occupancy limit of the shape; larger
 * requests are capped at it).  Recaptures the step graph. */
int fst_batch_set_tile(fst_batch* b, int width, int height, int blocks_per_sm);
int fst_batch_set_tile_height(fst_batch* b, int tile_height);  /* keeps width, blocks */
int fst_batch_info(const fst_batch* b, fst_batch_info_t* out);
/* Autotuner: time every tile shape (width x height above) at up to four
 * persistent blocks-per-SM counts (the occupancy limit and about 3/4, 1/2
 * and 1/4 of it) on this ensemble, 3 graph replays each after one warm-up
 * (state restored afterwards), and keep the fastest.  With json_path, reuse a
 * stored choice for the same GPU and ensemble signature unless `force`, and
 * store new ones with every candidate's ms per step.  fst_batch_info reports
 * the chosen and the slowest candidate's times. */
int fst_batch_tune(fst_batch* b, const char* json_path, int force);

/* Learned smoothness classifier (FST_MODE_HYBRID).  No counterpart in the
 * reference, which runs full WENO5 on every face (src/flux.hpp:223-310).
 *
 * A 20 -> 32 -> 32 -> 1 MLP (ReLU, ReLU, sigmoid) reads, per face, the five
 * undivided differences across the 6-cell WENO stencil of density,
 * pressure, face-normal velocity and the largest mass fraction, each
 * normalised by the sum of their magnitudes.  Inference runs in BF16 on the
 * tensor cores with FP32 accumulation; faces with output <= threshold take
 * the linear optimal-weight 5th-order upwind flux, the rest full WENO5.
 * Parameters are FP32, FST_MLP_PARAMS of them, packed as W1[32][20], b1[32],
 * W2[32][32], b2[32], w3[32], b3.
 * Labels come from WENO5 smoothness indicators: a face is non-smooth when,
 * for density or pressure on either upwind stencil, max(beta)/min(beta)
 * exceeds `label_ratio`. */
#define FST_MLP_IN 20
#define FST_MLP_HID 32
#define FST_MLP_PARAMS (FST_MLP_HID * FST_MLP_IN + FST_MLP_HID + FST_MLP_HID * FST_MLP_HID + \
                        FST_MLP_HID + FST_MLP_HID + 1)
/* Features (row-major [n][20] FP32, device) and labels (uint8, device) of
 * every face of the context's current state (3 faces per face index of the
 * face box); *count receives the number written (<= capacity).  The context
 * must be FST_MODE_MIXED or FST_MODE_HYBRID. */
int fst_hybrid_features(fst_ctx* ctx, float* d_features, unsigned char* d_labels,
                        size_t capacity, float label_ratio, size_t* count);
/* Loss and gradient of the mean binary cross-entropy (positives weighted by
 * pos_weight) over n samples, FP32 on the device (d_grad: FST_MLP_PARAMS). */
int fst_mlp_grad(const float* d_features, const unsigned char* d_labels, size_t n,
                 const float* d_params, float pos_weight, float* d_grad, float* h_loss,
                 void* cuda_stream);
/* One epoch of minibatch Adam over the n samples (sample order as given). */
int fst_mlp_train_epoch(const float* d_features, const unsigned char* d_labels, size_t n,
                        float* d_params, float* d_adam_m, float* d_adam_v, int* adam_step,
                        float lr, float pos_weight, int batch, float* h_mean_loss,
                        void* cuda_stream);
/* Classifier output probability per sample: FP32 CUDA-core path
 * (tensor_cores = 0) or the BF16 tensor-core inference path (1). */
int fst_mlp_forward(const float* d_features, size_t n, const float* d_params, float* d_out,
                    int tensor_cores, void* cuda_stream);
/* Install trained parameters (host FP32) in a hybrid context and set the
 * routing threshold; until then a hybrid context runs full WENO5. */
int fst_hybrid_set_params(fst_ctx* ctx, const float* params, float threshold);
/* Audit counters of a hybrid context: faces classified, faces routed to
 * WENO, and on audit steps (every fst_config.audit_every steps, run with
 * full WENO) faces labelled non-smooth and those the classifier would have
 * sent to the linear flux. */
typedef struct fst_hybrid_counts {
  int64_t faces, weno_faces, audit_faces, audit_nonsmooth, audit_missed;
} fst_hybrid_counts;
int fst_hybrid_get_counts(fst_ctx* ctx, fst_hybrid_counts* out, int reset);

/* Seeded initial conditions generated on the host (same on every platform;
 * no libm calls).  `kind`: FST_IC_*.  Writes the interior of U (LayoutLeft,
 * n = fst_state_size()); ghosts and C variables are set to zero. */
enum {
  FST_IC_SHOCK_TUBE_2D = 1,   /* Sod tube, diaphragm at x = 0.5            */
  FST_IC_EXPANSION_3D = 2,    /* high-pressure sphere of species 2 + noise */
  FST_IC_MIXING_3D = 3,       /* Gaussian pressure kernels + species blobs */
  FST_IC_RT_2D = 4,           /* Rayleigh-Taylor interface, Fourier modes  */
  FST_IC_RANDOM_SMOOTH = 5    /* smooth random fields (tests)              */
};
typedef struct fst_ic_params {
  int kind;
  uint64_t seed;
  double p_ambient, T_ambient;   /* Pa, K                                    */
  double p_high;                 /* expansion: bubble pressure             */
  double radius;                 /* expansion: bubble radius               */
  double noise;                  /* relative density noise amplitude       */
  double rho_heavy, rho_light;   /* RT                                     */
  int nkernels;                  /* mixing: number of pressure kernels     */
  int reserved[7];
} fst_ic_params;
int fst_fill_initial_conditions(const fst_config* cfg, const fst_ic_params* ic,
                                double* U, size_t n);

#ifdef __cplusplus
}
#endif
#endif /* FST_H */
