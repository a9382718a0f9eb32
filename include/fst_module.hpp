/*
 * fst_module.hpp — C++ host interface over the libfst C ABI (fst.h) that keeps
 * the shape of the reference's module classes: rk_func with its hooks
 * compute / preStep / postStep / preSim / postSim and the var, dvar, varx
 * arrays (src/rkfunction.hpp:36-69), the four modules cart2d_func,
 * cart3d_func, gen2d_func, gen3d_func (chosen as src/main.cpp:40-50 does),
 * applyBCs (src/bc.hpp:33) and rkAdvance (src/rk.hpp).  Header-only; link
 * against libfst.so.
 *
 * The reference keeps var/dvar/varx on the device and host code reaches them
 * through mirrors (create_mirror_view + deep_copy).  Here the state lives in
 * the library's context; `var`, `dvar` and `varx` are host mirrors with the
 * same LayoutLeft indexing, moved by upload() / download() (var), compute()
 * (dvar) and secondary() (varx).  Errors throw fst::Error with the
 * library's status code and message (the reference exits the process).
 */
#ifndef FST_MODULE_HPP
#define FST_MODULE_HPP

#include <cstddef>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "fst.h"

namespace fst {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code(code) {}
  int code;
};

// Host array with the reference's LayoutLeft indexing a(i, j, k, v).
class HostArray {
 public:
  HostArray() = default;
  HostArray(int n0, int n1, int n2, int n3)
      : n0_(n0), n1_(n1), n2_(n2), n3_(n3), data_((size_t)n0 * n1 * n2 * n3, 0.0) {}
  double& operator()(int i, int j, int k, int v) {
    return data_[(size_t)i + (size_t)n0_ * ((size_t)j + (size_t)n1_ * ((size_t)k + (size_t)n2_ * v))];
  }
  double operator()(int i, int j, int k, int v) const {
    return data_[(size_t)i + (size_t)n0_ * ((size_t)j + (size_t)n1_ * ((size_t)k + (size_t)n2_ * v))];
  }
  double* data() { return data_.data(); }
  const double* data() const { return data_.data(); }
  size_t size() const { return data_.size(); }
  int extent(int d) const { return d == 0 ? n0_ : d == 1 ? n1_ : d == 2 ? n2_ : n3_; }

 private:
  int n0_ = 0, n1_ = 0, n2_ = 0, n3_ = 0;
  std::vector<double> data_;
};

// The module base: one libfst context and the host mirrors.
class rk_func {
 public:
  explicit rk_func(const fst_config& cf) : cf_(cf) {
    int rc = fst_create(&cf_, &ctx_);
    if (rc != FST_OK) throw Error(rc, "fst_create failed (the reason is on stderr)");
    const int ngi = cf.nci + 2 * cf.ng, ngj = cf.ncj + 2 * cf.ng;
    const int ngk = cf.ndim == 3 ? cf.nck + 2 * cf.ng : 1;
    const int nvt = fst_nvt(&cf_);
    var = HostArray(ngi, ngj, ngk, nvt);
    dvar = HostArray(ngi, ngj, ngk, nvt);
    varx = HostArray(ngi, ngj, ngk, cf.ndim == 3 ? 6 : 5);
  }
  virtual ~rk_func() { fst_destroy(ctx_); }
  rk_func(const rk_func&) = delete;
  rk_func& operator=(const rk_func&) = delete;

  // The hooks of the reference's rk_func.  compute() leaves R(var) of the
  // device state in dvar (3D modules apply the BCs first, as
  // cart3d_func::compute does).  The time step itself is rkAdvance.
  virtual void compute() {
    check(fst_compute_rhs(ctx_, dvar.data(), dvar.size()), "compute");
  }
  virtual void preStep() {}   // 2D BCs run inside fst_rk_step
  // postStep's noise filter when the deck enables it (fiesta.noise, the
  // `if (cf.noise)` block of src/cart3d.cpp:319-374, src/cart2d.cpp:257-307,
  // src/gen2d.cpp:150-179).  The reference's other postStep work, the
  // secondary variables of an output step, is secondary() here, called by
  // the host when it writes.
  virtual void postStep() {
    if (noise_on_) check(fst_noise_filter(ctx_, &noise_), "postStep");
  }
  virtual void preSim() {}
  virtual void postSim() { check(fst_synchronize(ctx_), "postSim"); }

  // Host mirrors <-> device state (the deep_copy calls of the reference).
  void upload() { check(fst_set_state(ctx_, var.data(), var.size()), "upload"); }
  void download() { check(fst_get_state(ctx_, var.data(), var.size()), "download"); }
  // Secondary variables (velocity, p, T, rho) of the device state into varx.
  void secondary() { check(fst_secondary(ctx_, varx.data(), varx.size()), "secondary"); }

  // fiesta.noise.{dh, eta, coff, nt, mode} (src/input.cpp:270-277)
  virtual void set_noise(const fst_noise_params& np) {
    noise_ = np;
    noise_on_ = true;
  }

  fst_ctx* context() const { return ctx_; }
  const fst_config& config() const { return cf_; }

  HostArray var, dvar, varx;

 protected:
  void check(int rc, const char* what) const {
    if (rc != FST_OK) throw Error(rc, std::string(what) + ": " + fst_last_error(ctx_));
  }
  fst_config cf_;
  fst_ctx* ctx_ = nullptr;
  fst_noise_params noise_{};
  bool noise_on_ = false;
};

class cart3d_func : public rk_func {
 public:
  explicit cart3d_func(const fst_config& cf) : rk_func(require(cf)) {}

 private:
  static const fst_config& require(const fst_config& cf) {
    if (cf.ndim != 3 || cf.grid_type != FST_GRID_CARTESIAN)
      throw Error(FST_ERR_INVALID, "cart3d_func needs a 3D cartesian config");
    return cf;
  }
};

class cart2d_func : public rk_func {
 public:
  explicit cart2d_func(const fst_config& cf) : rk_func(require(cf)) {}
  // cart2d_func::preSim applies the BCs once (src/cart2d.cpp:136-145)
  void preSim() override { check(fst_apply_bcs(ctx_), "preSim"); }

 private:
  static const fst_config& require(const fst_config& cf) {
    if (cf.ndim != 2 || cf.grid_type != FST_GRID_CARTESIAN)
      throw Error(FST_ERR_INVALID, "cart2d_func needs a 2D cartesian config");
    return cf;
  }
};

// Generalized grids: node coordinates in `grid` (ni, nj, nk, 3), LayoutLeft,
// as loadGrid fills the module's view; preSim computes the metrics.
class gen_func : public rk_func {
 public:
  explicit gen_func(const fst_config& cf) : rk_func(require(cf)) {
    grid = HostArray(cf.nci + 1, cf.ncj + 1, cf.ndim == 3 ? cf.nck + 1 : 1, 3);
  }
  void preSim() override { check(fst_set_grid(ctx_, grid.data(), grid.size()), "preSim"); }
  HostArray grid;

 private:
  static const fst_config& require(const fst_config& cf) {
    if (cf.grid_type != FST_GRID_GENERALIZED)
      throw Error(FST_ERR_INVALID, "gen2d_func / gen3d_func need grid_type = generalized");
    return cf;
  }
};
class gen3d_func : public gen_func {
 public:
  explicit gen3d_func(const fst_config& cf) : gen_func(cf) {
    if (cf.ndim != 3) throw Error(FST_ERR_INVALID, "gen3d_func needs ndim = 3");
  }
  // gen3d_func::postStep has no noise filter (src/gen3d.cpp:111-128)
  void set_noise(const fst_noise_params&) override {}
};
class gen2d_func : public gen_func {
 public:
  explicit gen2d_func(const fst_config& cf) : gen_func(cf) {
    if (cf.ndim != 2) throw Error(FST_ERR_INVALID, "gen2d_func needs ndim = 2");
  }
};

// A config written by `python -m fiesta_gb300.deck <deck.lua> <prefix>`
// (<prefix>.cfg, the raw struct): the deck's keys, read by the library's
// Lua-subset reader, for a C++ host.
inline fst_config load_config(const std::string& path) {
  fst_config c;
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw Error(FST_ERR_INVALID, "cannot open " + path);
  const size_t got = std::fread(&c, 1, sizeof(c), f);
  const bool more = std::fgetc(f) != EOF;
  std::fclose(f);
  if (got != sizeof(c) || more) throw Error(FST_ERR_SIZE, path + " is not an fst_config");
  if (c.abi_version != FST_ABI_VERSION) throw Error(FST_ERR_INVALID, path + ": ABI version");
  return c;
}

// Raw FP64 array (<prefix>.U0, <prefix>.X) into a host mirror of its size.
inline void load_array(const std::string& path, HostArray& a) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw Error(FST_ERR_INVALID, "cannot open " + path);
  const size_t got = std::fread(a.data(), sizeof(double), a.size(), f);
  const bool more = std::fgetc(f) != EOF;
  std::fclose(f);
  if (got != a.size() || more) throw Error(FST_ERR_SIZE, path + ": size does not match");
}

// <prefix>.noise, the raw fst_noise_params the deck exporter writes when
// fiesta.noise.enabled is set; false when there is no such file.
inline bool load_noise(const std::string& path, fst_noise_params& np) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  const size_t got = std::fread(&np, 1, sizeof(np), f);
  const bool more = std::fgetc(f) != EOF;
  std::fclose(f);
  if (got != sizeof(np) || more) throw Error(FST_ERR_SIZE, path + " is not an fst_noise_params");
  return true;
}

// The module src/main.cpp:40-50 picks for a config.
inline std::unique_ptr<rk_func> make_module(const fst_config& cf) {
  if (cf.grid_type == FST_GRID_GENERALIZED) {
    if (cf.ndim == 3) return std::unique_ptr<rk_func>(new gen3d_func(cf));
    return std::unique_ptr<rk_func>(new gen2d_func(cf));
  }
  if (cf.ndim == 3) return std::unique_ptr<rk_func>(new cart3d_func(cf));
  return std::unique_ptr<rk_func>(new cart2d_func(cf));
}

// applyBCs(cf, f) (src/bc.cpp:179-249) on the device state.
inline void applyBCs(rk_func& f) {
  int rc = fst_apply_bcs(f.context());
  if (rc != FST_OK) throw Error(rc, std::string("applyBCs: ") + fst_last_error(f.context()));
}

// rkAdvance (src/rk.cpp:28-70) preceded by the module's preStep BCs:
// `nsteps` time steps of the device state.
inline void rkAdvance(rk_func& f, int nsteps = 1) {
  int rc = fst_rk_step(f.context(), nsteps);
  if (rc != FST_OK) throw Error(rc, std::string("rkAdvance: ") + fst_last_error(f.context()));
}

}  // namespace fst

#endif
