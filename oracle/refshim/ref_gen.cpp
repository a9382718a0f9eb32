// ref_gen.cpp — construction of the reference's gen2d_func / gen3d_func and
// access to their metric views, for oracle/_ref/libfiesta_ref.so.
// TEST INFRASTRUCTURE ONLY.
//
// Compiled without HAVE_MPI (the class layouts of src/gen2d.hpp and
// src/gen3d.hpp depend on it, so every use of the classes stays in this
// translation unit).  Without HAVE_MPI, preSim skips the metric halo
// exchange; on one rank with no periodic axis that exchange only writes
// zeros that the ghost mirrors then overwrite, so the metrics are the same.
#include <cstring>

#include "gen2d.hpp"
#include "gen3d.hpp"

rk_func* ref_new_gen(inputConfig& cf) {
  if (cf.ndim == 3) return new gen3d_func(cf);
  return new gen2d_func(cf);
}

size_t ref_gen_metrics(rk_func* f, int ndim, double* out, size_t n) {
  if (ndim == 3) {
    auto* g = dynamic_cast<gen3d_func*>(f);
    if (!g || g->metrics.size() != n) return 0;
    std::memcpy(out, g->metrics.data(), n * sizeof(double));
  } else {
    auto* g = dynamic_cast<gen2d_func*>(f);
    if (!g || g->metrics.size() != n) return 0;
    std::memcpy(out, g->metrics.data(), n * sizeof(double));
  }
  return n;
}

// gen2d_func's noise indicator (allocated by its constructor only when the
// deck enables the filter).
void ref_gen2d_noise_init(rk_func* f, int ngi, int ngj) {
  auto* g = dynamic_cast<gen2d_func*>(f);
  if (g && g->noise.size() == 0) g->noise = FS2D_I("noise", ngi, ngj);
}
int ref_gen2d_noise_at(rk_func* f, int i, int j) {
  auto* g = dynamic_cast<gen2d_func*>(f);
  return g && g->noise.size() ? g->noise(i, j) : 0;
}
