// Time steps through the C++ module interface (include/fst_module.hpp) for a
// cartesian 3D case and a generalized 2D case; writes the configs, inputs
// and results as raw files <prefix>_<case>.{cfg,X,U0,U1} for the test to
// compare with the oracle.
#include <cmath>
#include <cstdio>
#include <string>

#include "fst_module.hpp"

static void dump(const std::string& path, const void* p, size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f || std::fwrite(p, 1, bytes, f) != bytes) throw fst::Error(FST_ERR_INVALID, "write " + path);
  std::fclose(f);
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::printf("usage: module_step <output prefix>\n");
    return 2;
  }
  const std::string pre = argv[1];
  try {
    {  // cart3d_func: two species, viscous, C-equation, 2 steps
      fst_config c;
      fst_config_defaults(&c);
      c.ndim = 3;
      c.nci = 12; c.ncj = 10; c.nck = 8;
      c.dx = 1.0 / 12; c.dy = 1.0 / 10; c.dz = 1.0 / 8;
      c.dt = 2e-7;
      c.ns = 2;
      c.gamma[0] = 1.4; c.M[0] = 0.02896; c.mu[0] = 1.8e-5;
      c.gamma[1] = 1.67; c.M[1] = 0.004; c.mu[1] = 1.99e-5;
      c.visc = 1; c.ceq = 1; c.kap = 10.0; c.eps = 0.4; c.alpha = 40.0;
      fst::cart3d_func f(c);
      fst_ic_params ic{};
      ic.kind = FST_IC_MIXING_3D;
      ic.seed = 11;
      ic.p_ambient = 1e5;
      ic.T_ambient = 300.0;
      ic.nkernels = 3;
      if (fst_fill_initial_conditions(&c, &ic, f.var.data(), f.var.size()) != FST_OK)
        throw fst::Error(FST_ERR_INVALID, "initial conditions");
      dump(pre + "_cart3d.cfg", &c, sizeof(c));
      dump(pre + "_cart3d.U0", f.var.data(), f.var.size() * sizeof(double));
      f.upload();
      f.preSim();
      fst::rkAdvance(f, 2);
      f.postSim();
      f.download();
      dump(pre + "_cart3d.U1", f.var.data(), f.var.size() * sizeof(double));
    }
    {  // gen2d_func on a sine-perturbed channel, QUICK fluxes, 3 steps
      fst_config c;
      fst_config_defaults(&c);
      c.ndim = 2;
      c.nci = 16; c.ncj = 12; c.nck = 1;
      c.dx = c.dy = c.dz = 1.0;
      c.dt = 1e-4;
      c.R = 1.0;
      c.ns = 1;
      c.gamma[0] = 1.4; c.M[0] = 1.0;
      c.grid_type = FST_GRID_GENERALIZED;
      c.scheme = FST_SCHEME_QUICK;
      fst::gen2d_func f(c);
      for (int j = 0; j <= c.ncj; ++j)
        for (int i = 0; i <= c.nci; ++i) {
          const double x = i / 16.0, y0 = j / 12.0, dh = 0.02 * std::sin(6.283185307179586 * x);
          f.grid(i, j, 0, 0) = x;
          f.grid(i, j, 0, 1) = dh + (1.0 - dh) * y0;
        }
      fst_ic_params ic{};
      ic.kind = FST_IC_RANDOM_SMOOTH;
      ic.seed = 5;
      if (fst_fill_initial_conditions(&c, &ic, f.var.data(), f.var.size()) != FST_OK)
        throw fst::Error(FST_ERR_INVALID, "initial conditions");
      f.upload();
      fst::applyBCs(f);  // finite ghosts (the module itself never fills them)
      f.download();
      dump(pre + "_gen2d.cfg", &c, sizeof(c));
      dump(pre + "_gen2d.X", f.grid.data(), f.grid.size() * sizeof(double));
      dump(pre + "_gen2d.U0", f.var.data(), f.var.size() * sizeof(double));
      f.preSim();
      fst::rkAdvance(f, 3);
      f.download();
      dump(pre + "_gen2d.U1", f.var.data(), f.var.size() * sizeof(double));
    }
  } catch (const fst::Error& e) {
    std::printf("fst::Error %d: %s\n", e.code, e.what());
    return 1;
  }
  std::printf("module_step: ok\n");
  return 0;
}
