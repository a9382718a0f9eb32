// Runs a FIESTA deck with no Python: the Lua 5.3 VM reads it (fst_deck.h),
// the C++ module interface (fst_module.hpp) builds the module the reference's
// main would pick, loads fiesta.initial_conditions and steps it.
//
//   module_lua <deck.lua> <prefix> <steps>
//
// writes <prefix>.cfg (the raw fst_config) and <prefix>.U0 (the initial
// state, LayoutLeft FP64); with steps > 0 it also runs them on the GPU and
// writes <prefix>.U1.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "fst_deck.h"
#include "fst_module.hpp"

static void write(const std::string& path, const void* p, size_t bytes) {
  FILE* o = std::fopen(path.c_str(), "wb");
  if (!o || std::fwrite(p, 1, bytes, o) != bytes) throw fst::Error(FST_ERR_INVALID, "write " + path);
  std::fclose(o);
}

int main(int argc, char** argv) {
  if (argc != 4) {
    std::printf("usage: module_lua <deck.lua> <prefix> <steps>\n");
    return 2;
  }
  const std::string pre = argv[2];
  const int steps = std::atoi(argv[3]);
  char err[512];
  fst_deck* d = nullptr;
  int rc = fst_deck_load(argv[1], &d, err, sizeof(err));
  if (rc) {
    std::printf("fst_deck_load %d: %s\n", rc, err);
    return 1;
  }
  try {
    fst_config cf;
    if ((rc = fst_deck_config(d, &cf))) throw fst::Error(rc, fst_deck_last_error(d));
    write(pre + ".cfg", &cf, sizeof(cf));
    std::vector<double> X;
    if (cf.grid_type == FST_GRID_GENERALIZED) {
      X.resize((size_t)(cf.nci + 1) * (cf.ncj + 1) * (cf.ndim == 3 ? cf.nck + 1 : 1) * 3);
      if ((rc = fst_deck_grid_nodes(d, &cf, X.data(), X.size())))
        throw fst::Error(rc, fst_deck_last_error(d));
    }
    const int ng = cf.ng, nv = (cf.ndim == 3 ? 4 : 3) + cf.ns, nvt = nv + (cf.ceq ? 5 : 0);
    const size_t n = (size_t)(cf.nci + 2 * ng) * (cf.ncj + 2 * ng) *
                     (cf.ndim == 3 ? cf.nck + 2 * ng : 1) * nvt;
    std::vector<double> U(n);
    if ((rc = fst_deck_initial_conditions(d, &cf, X.empty() ? nullptr : X.data(), U.data(), n)))
      throw fst::Error(rc, fst_deck_last_error(d));
    write(pre + ".U0", U.data(), n * sizeof(double));
    if (steps > 0) {
      auto f = fst::make_module(cf);
      fst_noise_params np;
      int noise = 0;
      fst_deck_noise(d, &np, &noise);
      if (noise) f->set_noise(np);
      for (size_t q = 0; q < n; ++q) f->var.data()[q] = U[q];
      if (auto* g = dynamic_cast<fst::gen_func*>(f.get()))
        for (size_t q = 0; q < X.size(); ++q) g->grid.data()[q] = X[q];
      f->upload();
      f->preSim();
      for (int t = 0; t < steps; ++t) {
        f->preStep();
        fst::rkAdvance(*f);
        f->postStep();
      }
      f->postSim();
      f->download();
      write(pre + ".U1", f->var.data(), n * sizeof(double));
    }
  } catch (const fst::Error& e) {
    std::printf("fst::Error %d: %s\n", e.code, e.what());
    fst_deck_destroy(d);
    return 1;
  }
  fst_deck_destroy(d);
  std::printf("module_lua: ok\n");
  return 0;
}
