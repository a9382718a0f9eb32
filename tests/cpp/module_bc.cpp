// Boundary-condition known answers through the C++ module interface
// (include/fst_module.hpp): the values the reference's tests/bc_outflow.cpp,
// tests/bc_reflective.cpp, tests/bc_hydrostatic.cpp and the periodic case of
// tests/test.cpp assert, on the same grids with three ghost layers.  Exit
// status 0 when every check holds.
#include <cstdio>

#include "fst_module.hpp"

static int failures = 0;
#define CHECK(cond)                                                  \
  do {                                                               \
    if (!(cond)) {                                                   \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);  \
      ++failures;                                                    \
    }                                                                \
  } while (0)

static fst_config kat_config(int bc, int nck = 3) {
  fst_config c;
  fst_config_defaults(&c);
  c.ndim = 3;
  c.nci = c.ncj = 3;
  c.nck = nck;
  c.dx = c.dy = c.dz = 1.0;
  c.dt = 1.0;
  c.R = 1.0;
  c.ns = 1;
  c.gamma[0] = 1.4;
  c.M[0] = 1.0;
  c.mu[0] = 1.0;
  c.bc_xmin = c.bc_xmax = c.bc_ymin = c.bc_ymax = c.bc_zmin = c.bc_zmax = bc;
  return c;
}

int main() {
  try {
    {  // outflow: a mirror of the interior into the ghosts, x-y plane
      fst::cart3d_func f(kat_config(FST_BC_OUTFLOW));
      int val = 1;
      for (int j = 3; j <= 5; ++j)
        for (int i = 3; i <= 5; ++i) f.var(i, j, 3, 0) = val++;
      f.upload();
      fst::applyBCs(f);
      f.download();
      CHECK(f.var(4, 0, 3, 0) == 8);
      CHECK(f.var(0, 4, 3, 0) == 6);
      CHECK(f.var(4, 8, 3, 0) == 2);
      CHECK(f.var(8, 4, 3, 0) == 4);
      CHECK(f.var(0, 0, 3, 0) == 9);
      CHECK(f.var(8, 0, 3, 0) == 7);
      CHECK(f.var(0, 8, 3, 0) == 3);
      CHECK(f.var(8, 8, 3, 0) == 1);
    }
    {  // reflective: the mirror with the normal momentum's sign flipped
      fst::cart3d_func f(kat_config(FST_BC_REFLECTIVE));
      int val = 1;
      for (int j = 3; j <= 5; ++j)
        for (int i = 3; i <= 5; ++i) {
          f.var(i, j, 3, 0) = val;
          f.var(i, j, 3, 1) = val++;
        }
      f.upload();
      fst::applyBCs(f);
      f.download();
      CHECK(f.var(4, 0, 3, 0) == 8 && f.var(4, 0, 3, 1) == -8);
      CHECK(f.var(0, 4, 3, 0) == -6 && f.var(0, 4, 3, 1) == 6);
      CHECK(f.var(4, 8, 3, 0) == 2 && f.var(4, 8, 3, 1) == -2);
      CHECK(f.var(8, 4, 3, 0) == -4 && f.var(8, 4, 3, 1) == 4);
    }
    {  // hydrostatic in y: energy extrapolated from the first two interior rows
      fst_config c = kat_config(FST_BC_OUTFLOW);
      c.bc_ymin = c.bc_ymax = FST_BC_HYDROSTATIC;
      fst::cart3d_func f(c);
      int val = 1;
      for (int j = 3; j <= 5; ++j)
        for (int i = 3; i <= 5; ++i) {
          f.var(i, j, 4, 3) = val++;
          f.var(i, j, 4, 4) = 1.0;
        }
      f.upload();
      fst::applyBCs(f);
      f.download();
      CHECK(f.var(4, 2, 4, 3) == -1 && f.var(4, 0, 4, 3) == -7 && f.var(0, 4, 4, 3) == 6);
      CHECK(f.var(4, 8, 4, 3) == 17 && f.var(8, 4, 4, 3) == 4);
      CHECK(f.var(0, 0, 4, 3) == -6 && f.var(8, 0, 4, 3) == -8);
      CHECK(f.var(0, 8, 4, 3) == 18 && f.var(8, 8, 4, 3) == 16);
    }
    {  // periodic in x, y, z on a 3x3x10 interior
      fst_config c = kat_config(FST_BC_REFLECTIVE, 10);
      c.xper = c.yper = c.zper = 1;
      fst::cart3d_func f(c);
      for (int k = 3; k < 13; ++k) f.var(4, 4, k, 0) = 47 + k;  // 50 .. 59
      f.upload();
      fst::applyBCs(f);
      f.download();
      CHECK(f.var(4, 4, 0, 0) == 57 && f.var(4, 4, 1, 0) == 58 && f.var(4, 4, 2, 0) == 59);
      CHECK(f.var(4, 4, 13, 0) == 50 && f.var(4, 4, 14, 0) == 51 && f.var(4, 4, 15, 0) == 52);
    }
    {  // the module choice and a rejected config
      fst_config c = kat_config(FST_BC_OUTFLOW);
      auto m = fst::make_module(c);
      CHECK(dynamic_cast<fst::cart3d_func*>(m.get()) != nullptr);
      c.ndim = 2;
      bool threw = false;
      try {
        fst::cart3d_func bad(c);
      } catch (const fst::Error& e) {
        threw = e.code == FST_ERR_INVALID;
      }
      CHECK(threw);
    }
  } catch (const fst::Error& e) {
    std::printf("fst::Error %d: %s\n", e.code, e.what());
    return 2;
  }
  std::printf("%s\n", failures ? "module_bc: FAILED" : "module_bc: ok");
  return failures ? 1 : 0;
}
