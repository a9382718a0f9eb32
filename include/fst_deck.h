/*
 * fst_deck.h — FIESTA's Lua input deck read by the Lua 5.3 C API, for C and
 * C++ hosts that run the library without Python.
 *
 * The deck runs in a Lua state exactly as the reference's luaReader sets it
 * up (src/luaReader.cpp:39-76: a global table `fiesta` with the sub-tables
 * ceq, noise, restart, bc, time, viscosity, buoyancy, grid, mpi, hdf5, eos,
 * progress and status, then luaL_openlibs and the file); the keys of the
 * right-hand-side path are read with the reference's conversions
 * (luaReader::get / getValue / getArray, src/luaReader.cpp:78-161, 352-400;
 * executeConfiguration, src/input.cpp:136-308; the species list,
 * src/luaReader.cpp:163-209), and fiesta.initial_conditions /
 * fiesta.initialize_grid are called per cell / node as
 * loadInitialConditions and loadGrid do (src/input.cpp:445-560).  The
 * library's own keys live in `fiesta.gb300` (mode = "plain" | "mixed" |
 * "hybrid", audit_every, classify_every).
 *
 * Library: fiesta_gb300/libfst_deck.so, built against the Lua 5.3 sources of
 * a FIESTA tree (tpls/lua/src) by fiesta_gb300/build.py (build_deck).
 * Errors return the FST_ERR_* codes of fst.h and fill a message.
 */
#ifndef FST_DECK_H
#define FST_DECK_H

#include <stddef.h>

#include "fst.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fst_deck fst_deck;

/* Run the deck at `path` and read its keys.  On failure *out is NULL and
 * `err` (errlen bytes, may be NULL) receives the message. */
int fst_deck_load(const char* path, fst_deck** out, char* err, size_t errlen);
void fst_deck_destroy(fst_deck* d);
const char* fst_deck_last_error(const fst_deck* d);

/* The run configuration (cf. the reference's inputConfig). */
int fst_deck_config(const fst_deck* d, fst_config* cfg);
/* fiesta.noise: *enabled = 0 when the filter is off (or the module has none,
 * the generalized 3D one); otherwise the parameters. */
int fst_deck_noise(const fst_deck* d, fst_noise_params* np, int* enabled);
/* Node coordinates of a generalized grid, n = fst_grid_size(cfg):
 * fiesta.initialize_grid(i, j, k, v) at every node for v < ndim (loadGrid,
 * src/input.cpp:529-560), LayoutLeft (ni, nj, nk, 3). */
int fst_deck_grid_nodes(fst_deck* d, const fst_config* cfg, double* X, size_t n);
/* The initial state, n = fst_state_size(cfg): fiesta.initial_conditions(x,
 * y, z, v) at every interior cell centre for v < nv (uniform grids: x =
 * dx*(i-ng) + dx/2; generalized grids: the mean of the cell's nodes X);
 * ghosts and C-equation variables zero. */
int fst_deck_initial_conditions(fst_deck* d, const fst_config* cfg, const double* X,
                                double* U, size_t n);

#ifdef __cplusplus
}  // extern "C"
#endif

#endif
