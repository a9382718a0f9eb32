// ref_harness.cpp — C entry points around the reference's own cart2d_func /
// cart3d_func / gen2d_func / gen3d_func / applyBCs / rkAdvance, compiled from
// the reference sources by oracle/ref_build.sh into
// oracle/_ref/libfiesta_ref.so.
//
// TEST INFRASTRUCTURE ONLY: it produces the golden vectors under tests/golden
// and cross-checks the oracle restatement; nothing in the product loads it.
//
// The time loop mirrors src/main.cpp:61-72 / Fiesta::step
// (src/fiesta.cpp:333-340): preStep, rkAdvance, postStep, t += 1.
#include <omp.h>

#include <cstring>
#include <memory>

#include "cart2d.hpp"
#include "cart3d.hpp"
#include "rk.hpp"

#include "../../include/fst.h"

// Diagnostics is only exercised with --diagnostics; these empty bodies stand
// in for src/diagnostics.cpp, which needs the fmt-based logger.
Diagnostics::Diagnostics() {}
Diagnostics::Diagnostics(size_t, size_t, size_t, size_t, size_t, int) {}
Diagnostics::Diagnostics(Diagnostics&&) {}
Diagnostics& Diagnostics::operator=(const Diagnostics&) { return *this; }
Diagnostics& Diagnostics::operator=(Diagnostics&&) { return *this; }
void Diagnostics::init(size_t, FS4D&) {}
void Diagnostics::start(size_t, FS4D&) {}
void Diagnostics::stop(std::string, size_t, FS4D&, std::map<std::string, FS4D>&) {}
void Diagnostics::finalize(size_t, FS4D&, std::map<std::string, FS4D>&) {}

namespace {
BCType bc_of(int t) {
  switch (t) {
    case FST_BC_REFLECTIVE: return BCType::reflective;
    case FST_BC_NOSLIP: return BCType::noslip;
    case FST_BC_HYDROSTATIC: return BCType::hydrostatic;
    default: return BCType::outflow;
  }
}
}  // namespace

struct ref_ctx {
  inputConfig cf;
  std::unique_ptr<rk_func> f;
};

// ref_gen.cpp
rk_func* ref_new_gen(inputConfig& cf);
size_t ref_gen_metrics(rk_func* f, int ndim, double* out, size_t n);
void ref_gen2d_noise_init(rk_func* f, int ngi, int ngj);
int ref_gen2d_noise_at(rk_func* f, int i, int j);

extern "C" {

int ref_create(const fst_config* c, ref_ctx** out) {
  ref_ctx* x = new ref_ctx();
  inputConfig& cf = x->cf;
  // executeConfiguration's derived fields (src/input.cpp:330-435)
  cf.ndim = c->ndim;
  cf.ng = c->ng;
  cf.nci = c->nci;
  cf.ncj = c->ncj;
  cf.nck = c->ndim == 3 ? c->nck : 1;
  cf.ngi = cf.nci + 2 * cf.ng;
  cf.ngj = cf.ncj + 2 * cf.ng;
  cf.ngk = c->ndim == 3 ? cf.nck + 2 * cf.ng : 1;
  cf.ni = cf.nci + 1;
  cf.nj = cf.ncj + 1;
  cf.nk = c->ndim == 3 ? cf.nck + 1 : 1;
  cf.ns = c->ns;
  cf.nv = (c->ndim == 3 ? 4 : 3) + cf.ns;
  cf.ceq = c->ceq != 0;
  cf.nvt = cf.nv + (cf.ceq ? 5 : 0);
  cf.dx = c->dx;
  cf.dy = c->dy;
  cf.dz = c->ndim == 3 ? c->dz : c->dx;
  cf.dt = c->dt;
  cf.R = c->R;
  for (int s = 0; s < cf.ns; ++s) {
    cf.speciesName.push_back("S" + std::to_string(s));
    cf.gamma.push_back(c->gamma[s]);
    cf.M.push_back(c->M[s]);
    cf.mu.push_back(c->mu[s]);
  }
  cf.visc = c->visc != 0;
  cf.kap = c->kap;
  cf.eps = c->eps;
  cf.alpha = c->alpha;
  cf.buoyancy = c->buoyancy != 0;
  cf.gAccel = c->g_accel;
  cf.rhoRef = c->rho_ref;
  cf.xPer = c->xper != 0;
  cf.yPer = c->yper != 0;
  cf.zPer = c->ndim == 3 ? c->zper != 0 : false;
  cf.bcL = bc_of(c->bc_xmin);
  cf.bcR = bc_of(c->bc_xmax);
  cf.bcB = bc_of(c->bc_ymin);
  cf.bcT = bc_of(c->bc_ymax);
  cf.bcH = c->ndim == 3 ? bc_of(c->bc_zmin) : BCType::outflow;
  cf.bcF = c->ndim == 3 ? bc_of(c->bc_zmax) : BCType::outflow;
  cf.xMinus = cf.xPlus = -1 + (int)cf.xPer;
  cf.yMinus = cf.yPlus = -1 + (int)cf.yPer;
  cf.zMinus = cf.zPlus = -1 + (int)cf.zPer;
  cf.t = 0;
  cf.scheme = c->scheme > 0 ? c->scheme : 1;  // src/input.cpp:317-323
  cf.grid = c->grid_type;
  // module choice of src/main.cpp:40-50
  if (cf.grid > 0) x->f.reset(ref_new_gen(cf));
  else if (c->ndim == 3) x->f.reset(new cart3d_func(cf));
  else x->f.reset(new cart2d_func(cf));
  *out = x;
  return 0;
}

void ref_destroy(ref_ctx* x) { delete x; }

int ref_set_state(ref_ctx* x, const double* U, size_t n) {
  if (n != x->f->var.size()) return FST_ERR_SIZE;
  std::memcpy(x->f->var.data(), U, n * sizeof(double));
  return 0;
}
int ref_get_state(ref_ctx* x, double* U, size_t n) {
  if (n != x->f->var.size()) return FST_ERR_SIZE;
  std::memcpy(U, x->f->var.data(), n * sizeof(double));
  return 0;
}
// loadGrid's copy into f->grid (src/input.cpp:529-560), then preSim, which
// computes the metrics (src/gen3d.cpp:129-335, src/gen2d.cpp:190-320).
int ref_set_grid(ref_ctx* x, const double* X, size_t n) {
  if (x->cf.grid == 0) return FST_ERR_UNSUPPORTED;
  if (n != x->f->grid.size()) return FST_ERR_SIZE;
  std::memcpy(x->f->grid.data(), X, n * sizeof(double));
  x->f->preSim();
  return 0;
}
int ref_get_metrics(ref_ctx* x, double* out, size_t n) {
  if (x->cf.grid == 0) return FST_ERR_UNSUPPORTED;
  return ref_gen_metrics(x->f.get(), x->cf.ndim, out, n) == n ? 0 : FST_ERR_SIZE;
}
int ref_apply_bcs(ref_ctx* x) {
  applyBCs(x->cf, x->f.get());
  return 0;
}
int ref_compute_rhs(ref_ctx* x, double* R, size_t n) {
  x->f->compute();
  if (R) {
    if (n != x->f->dvar.size()) return FST_ERR_SIZE;
    std::memcpy(R, x->f->dvar.data(), n * sizeof(double));
  }
  return 0;
}
int ref_rk_step(ref_ctx* x, int nsteps) {
  for (int s = 0; s < nsteps; ++s) {
    x->f->preStep();
    rkAdvance(x->cf, x->f);
    x->f->postStep();
    x->cf.t += 1;
  }
  return 0;
}
int ref_secondary(ref_ctx* x, double* out, size_t n) {
  x->cf.ioThisStep = true;  // postStep computes varx (src/cart3d.cpp:300-318)
  x->f->postStep();
  x->cf.ioThisStep = false;
  FS4D& vx = x->f->varx;
  size_t nc = (size_t)x->cf.ngi * x->cf.ngj * x->cf.ngk;
  size_t nf = x->cf.ndim == 3 ? 6 : 5;
  if (n != nc * nf) return FST_ERR_SIZE;
  std::memcpy(out, vx.data(), n * sizeof(double));
  return 0;
}

// postStep with the noise filter on (src/cart3d.cpp:300-374,
// src/cart2d.cpp:239-307), its kernels run on one thread: the removal
// updates var in place while neighbours read it, so only the serial loop
// order gives a defined result.
int ref_noise_filter(ref_ctx* x, const fst_noise_params* np) {
  inputConfig& cf = x->cf;
  if (cf.grid > 0 && cf.ndim == 3) return FST_ERR_UNSUPPORTED;  // gen3d: no noise filter
  cf.noise = true;
  cf.n_dh = np->dh;
  cf.n_eta = np->eta;
  cf.n_coff = np->coff;
  cf.n_nt = np->nt;
  cf.n_mode = np->mode;
  if (cf.grid > 0) {  // gen2d_func::postStep (src/gen2d.cpp:150-179)
    ref_gen2d_noise_init(x->f.get(), cf.ngi, cf.ngj);
  } else if (cf.ndim == 3) {
    auto* f = dynamic_cast<cart3d_func*>(x->f.get());
    if (f->noise.size() == 0) f->noise = FS3D_I("noise", cf.ngi, cf.ngj, cf.ngk);
  } else {
    auto* f = dynamic_cast<cart2d_func*>(x->f.get());
    if (f->noise.size() == 0) f->noise = FS2D_I("noise", cf.ngi, cf.ngj);
  }
  const int nth = omp_get_max_threads();
  omp_set_num_threads(1);
  x->f->postStep();
  omp_set_num_threads(nth);
  cf.noise = false;
  return 0;
}
int ref_get_noise(ref_ctx* x, int* out, size_t n) {
  const inputConfig& cf = x->cf;
  if (n != (size_t)cf.ngi * cf.ngj * cf.ngk) return FST_ERR_SIZE;
  for (int k = 0; k < cf.ngk; ++k)
    for (int j = 0; j < cf.ngj; ++j)
      for (int i = 0; i < cf.ngi; ++i) {
        int v = 0;
        if (cf.grid > 0) {
          v = ref_gen2d_noise_at(x->f.get(), i, j);
        } else if (cf.ndim == 3) {
          auto* f = dynamic_cast<cart3d_func*>(x->f.get());
          if (f->noise.size()) v = f->noise(i, j, k);
        } else {
          auto* f = dynamic_cast<cart2d_func*>(x->f.get());
          if (f->noise.size()) v = f->noise(i, j);
        }
        out[(size_t)i + (size_t)cf.ngi * (j + (size_t)cf.ngj * k)] = v;
      }
  return 0;
}

}  // extern "C"
