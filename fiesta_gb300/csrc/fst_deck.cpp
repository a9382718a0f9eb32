// fst_deck.cpp — the reference's Lua input deck on the Lua 5.3 C API
// (include/fst_deck.h).  Host code only; built into libfst_deck.so together
// with the Lua sources of a FIESTA tree (tpls/lua/src).
//
// What is read and how mirrors the reference's input stage: the state set up
// by the luaReader constructor (src/luaReader.cpp:39-76), required keys and
// keys with defaults (luaReader::get, src/luaReader.cpp:78-161) with its
// conversions (getValue / getArray, src/luaReader.cpp:352-400: numbers by
// lua_tonumberx, ints by lua_tointegerx, bools by lua_toboolean, strings when
// lua_isstring), the keys of executeConfiguration (src/input.cpp:136-308),
// the species table (getSpeciesData, src/luaReader.cpp:163-209) and the
// per-cell / per-node calls of loadInitialConditions and loadGrid
// (src/input.cpp:445-560; luaReader::call, src/luaReader.cpp:317-345).
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

extern "C" {
#include "lauxlib.h"
#include "lua.h"
#include "lualib.h"
}

#include "../../include/fst_deck.h"

struct fst_deck {
  lua_State* L = nullptr;
  std::string filename, error;
  fst_config cf{};
  bool noise = false, gen3d = false;
  fst_noise_params np{};
};

namespace {

struct DeckError {
  int code;
  std::string msg;
};

const char* kPreset[] = {"ceq",       "noise", "restart", "bc",  "time",     "viscosity", "buoyancy",
                         "grid",      "mpi",   "hdf5",    "eos", "progress", "status"};

// Push fiesta.<keys...> (or nil); returns whether every level was found.
bool push_key(lua_State* L, std::initializer_list<const char*> keys) {
  lua_getglobal(L, "fiesta");
  for (const char* k : keys) {
    if (!lua_istable(L, -1)) {
      lua_pushnil(L);
      return false;
    }
    lua_getfield(L, -1, k);
    lua_remove(L, -2);
    if (lua_isnoneornil(L, -1)) return false;
  }
  return true;
}

std::string full(std::initializer_list<const char*> keys) {
  std::string s = "fiesta";
  for (const char* k : keys) s += std::string(".") + k;
  return s;
}

struct Reader {
  lua_State* L;
  std::string filename;

  [[noreturn]] void missing(std::initializer_list<const char*> keys) {
    throw DeckError{FST_ERR_INVALID, "Could not find required parameter '" + full(keys) +
                                         "' in '" + filename + "'"};
  }
  // luaReader::get without / with a default
  double num(std::initializer_list<const char*> keys) {
    const int top = lua_gettop(L);
    if (!push_key(L, keys)) {
      lua_settop(L, top);
      missing(keys);
    }
    int isnum;
    const double v = lua_tonumberx(L, -1, &isnum);
    lua_settop(L, top);
    return v;
  }
  double num(std::initializer_list<const char*> keys, double d) {
    const int top = lua_gettop(L);
    double v = d;
    if (push_key(L, keys)) {
      int isnum;
      v = lua_tonumberx(L, -1, &isnum);
    }
    lua_settop(L, top);
    return v;
  }
  long long integer(std::initializer_list<const char*> keys, long long d) {
    const int top = lua_gettop(L);
    long long v = d;
    if (push_key(L, keys)) {
      int isnum;
      v = (long long)lua_tointegerx(L, -1, &isnum);
    }
    lua_settop(L, top);
    return v;
  }
  bool boolean(std::initializer_list<const char*> keys, bool d) {
    const int top = lua_gettop(L);
    bool v = d;
    if (push_key(L, keys)) v = lua_toboolean(L, -1) != 0;
    lua_settop(L, top);
    return v;
  }
  std::string str(std::initializer_list<const char*> keys, const char* d = nullptr) {
    const int top = lua_gettop(L);
    const bool found = push_key(L, keys);
    if (!found && !d) {
      lua_settop(L, top);
      missing(keys);
    }
    std::string v = found ? "" : d;
    if (found && lua_isstring(L, -1)) v = lua_tostring(L, -1);
    lua_settop(L, top);
    return v;
  }
  // getArray: entries 1..n as numbers (lua_tonumberx, 0 when not a number)
  std::vector<double> array(std::initializer_list<const char*> keys, int n) {
    const int top = lua_gettop(L);
    if (!push_key(L, keys)) {
      lua_settop(L, top);
      missing(keys);
    }
    if (!lua_istable(L, -1)) {
      lua_settop(L, top);
      throw DeckError{FST_ERR_INVALID, full(keys) + " is not a table"};
    }
    std::vector<double> out;
    for (int i = 0; i < n; ++i) {
      lua_rawgeti(L, -1, i + 1);
      int isnum;
      out.push_back(lua_tonumberx(L, -1, &isnum));
      lua_pop(L, 1);
    }
    lua_settop(L, top);
    return out;
  }
};

std::string squash(std::string s) {
  std::string o;
  for (char ch : s)
    if (ch != '-' && ch != '_' && ch != ' ') o += (char)std::tolower((unsigned char)ch);
  return o;
}

// parseBC (src/bc.cpp:251-270)
int parse_bc(const std::string& name) {
  const std::string k = squash(name);
  if (k == "outflow") return FST_BC_OUTFLOW;
  if (k == "reflective") return FST_BC_REFLECTIVE;
  if (k == "noslip") return FST_BC_NOSLIP;
  if (k == "hydrostatic") return FST_BC_HYDROSTATIC;
  throw DeckError{FST_ERR_INVALID, "Unknown boundary condition '" + name + "'"};
}

void read_config(fst_deck* d) {
  Reader rd{d->L, d->filename};
  fst_config& c = d->cf;
  std::memset(&c, 0, sizeof(c));
  c.abi_version = FST_ABI_VERSION;
  (void)rd.str({"title"});
  const long long nt = rd.integer({"time", "nt"}, 0);
  c.dt = rd.num({"time", "dt"});
  if (nt == 0) (void)rd.integer({"time", "tend"}, 0);
  c.R = rd.num({"eos", "R"}, 8.314462);
  c.ndim = (int)rd.integer({"grid", "ndim"}, 2);
  if (c.ndim != 2 && c.ndim != 3)
    throw DeckError{FST_ERR_INVALID, "fiesta.grid.ndim must be 2 or 3"};
  c.visc = rd.boolean({"viscosity", "enabled"}, false);
  c.ng = (int)rd.integer({"ng"}, 3);
  const bool xper = rd.boolean({"bc", "xperiodic"}, false);
  const bool yper = rd.boolean({"bc", "yperiodic"}, false);
  const std::string scheme = rd.str({"advection_scheme"}, "weno5");
  const std::string grid = rd.str({"grid", "type"}, "cartesian");
  const std::vector<double> dx = rd.array({"grid", "dx"}, c.ndim);
  if (grid == "terrain" && c.ndim == 3) {  // src/input.cpp:294-302
    (void)rd.num({"tdx"});
    (void)rd.num({"tdy"});
    (void)rd.num({"h"});
  }
  const std::vector<double> ni = rd.array({"grid", "ni"}, c.ndim);
  (void)rd.array({"mpi", "procs"}, c.ndim);
  int bcs[6] = {FST_BC_OUTFLOW, FST_BC_OUTFLOW, FST_BC_OUTFLOW,
                FST_BC_OUTFLOW, FST_BC_OUTFLOW, FST_BC_OUTFLOW};
  if (!xper) {
    bcs[0] = parse_bc(rd.str({"bc", "xmin"}));
    bcs[1] = parse_bc(rd.str({"bc", "xmax"}));
  }
  if (!yper) {
    bcs[2] = parse_bc(rd.str({"bc", "ymin"}));
    bcs[3] = parse_bc(rd.str({"bc", "ymax"}));
  }
  c.buoyancy = rd.boolean({"buoyancy", "enabled"}, false);
  if (c.buoyancy) {
    c.g_accel = rd.num({"buoyancy", "acceleration"}, 9.81);
    c.rho_ref = rd.num({"buoyancy", "rho_reference"}, 0.0);
  }
  c.ceq = rd.boolean({"ceq", "enabled"}, false);
  if (c.ceq) {
    c.kap = rd.num({"ceq", "kappa"}, 1.23456);
    c.eps = rd.num({"ceq", "epsilon"});
    c.alpha = rd.num({"ceq", "alpha"});
    (void)rd.num({"ceq", "beta"});
    (void)rd.num({"ceq", "betae"});
  }
  d->noise = rd.boolean({"noise", "enabled"}, false);
  if (d->noise) {  // src/input.cpp:270-277
    d->np.dh = rd.num({"noise", "dh"});
    d->np.eta = rd.num({"noise", "eta"});
    d->np.coff = rd.num({"noise", "coff"});
    d->np.nt = (int)rd.integer({"noise", "nt"}, 1);
    d->np.mode = (int)rd.integer({"noise", "mode"}, 1);
  }
  bool zper = false;
  if (c.ndim == 3) {
    zper = rd.boolean({"bc", "zperiodic"}, false);
    if (!zper) {
      bcs[4] = parse_bc(rd.str({"bc", "zmin"}));
      bcs[5] = parse_bc(rd.str({"bc", "zmax"}));
    }
  }
  c.xper = xper;
  c.yper = yper;
  c.zper = zper;
  c.bc_xmin = bcs[0];
  c.bc_xmax = bcs[1];
  c.bc_ymin = bcs[2];
  c.bc_ymax = bcs[3];
  c.bc_zmin = bcs[4];
  c.bc_zmax = bcs[5];
  // species (src/luaReader.cpp:163-209)
  lua_State* L = d->L;
  const int top = lua_gettop(L);
  if (!push_key(L, {"species"})) {
    lua_settop(L, top);
    throw DeckError{FST_ERR_INVALID, "Could not find fiesta.species in '" + d->filename + "'"};
  }
  if (!lua_istable(L, -1)) {
    lua_settop(L, top);
    throw DeckError{FST_ERR_INVALID, "Error Reading Input File: Could not read blocks."};
  }
  const int ns = (int)lua_rawlen(L, -1);
  if (ns < 1) throw DeckError{FST_ERR_INVALID, "fiesta.species is empty"};
  if (ns > FST_MAX_SPECIES)
    throw DeckError{FST_ERR_UNSUPPORTED, "at most " + std::to_string(FST_MAX_SPECIES) +
                                             " species"};
  c.ns = ns;
  for (int s = 0; s < ns; ++s) {
    lua_rawgeti(L, -1, s + 1);
    if (!lua_istable(L, -1))
      throw DeckError{FST_ERR_INVALID, "fiesta.species[" + std::to_string(s + 1) +
                                           "] is not a table"};
    double* dst[3] = {&c.gamma[s], &c.M[s], &c.mu[s]};
    const char* names[3] = {"gamma", "M", "mu"};
    for (int q = 0; q < 3; ++q) {
      lua_getfield(L, -1, names[q]);
      int isnum;
      *dst[q] = lua_tonumberx(L, -1, &isnum);
      lua_pop(L, 1);
    }
    lua_pop(L, 1);
  }
  lua_settop(L, top);
  // this library's keys
  c.mode = FST_MODE_PLAIN_FP64;
  c.audit_every = 0;
  c.classify_every = 1;
  if (push_key(L, {"gb300"}) && lua_istable(L, -1)) {
    lua_getfield(L, -1, "mode");
    if (!lua_isnil(L, -1)) {
      std::string m = "?";
      if (lua_type(L, -1) == LUA_TSTRING) {
        m = lua_tostring(L, -1);
        std::transform(m.begin(), m.end(), m.begin(),
                       [](unsigned char ch) { return (char)std::tolower(ch); });
      }
      if (m == "plain" || m == "fp64") c.mode = FST_MODE_PLAIN_FP64;
      else if (m == "mixed") c.mode = FST_MODE_MIXED;
      else if (m == "hybrid") c.mode = FST_MODE_HYBRID;
      else throw DeckError{FST_ERR_INVALID, "fiesta.gb300.mode must be plain, mixed or hybrid"};
    }
    lua_pop(L, 1);
    lua_getfield(L, -1, "audit_every");
    if (!lua_isnil(L, -1)) {
      int isnum;
      c.audit_every = (int)lua_tointegerx(L, -1, &isnum);
    }
    lua_pop(L, 1);
    lua_getfield(L, -1, "classify_every");
    if (!lua_isnil(L, -1)) {
      int isnum;
      c.classify_every = (int)lua_tointegerx(L, -1, &isnum);
    }
    lua_pop(L, 1);
  }
  lua_settop(L, top);
  // sizes and spacings; generalized grids run in computational space
  // (dx = dy = dz = 1, src/input.cpp:344-350)
  const bool gen = grid == "generalized" || grid == "terrain";
  if (grid == "terrain" && c.ndim != 3)
    throw DeckError{FST_ERR_INVALID, "ndim must be equal to 3 for terrain"};
  if (grid != "cartesian" && !gen)
    throw DeckError{FST_ERR_INVALID, "unknown fiesta.grid.type '" + grid + "'"};
  c.grid_type = gen ? FST_GRID_GENERALIZED : FST_GRID_CARTESIAN;
  c.nci = (int)(long long)ni[0];
  c.ncj = (int)(long long)ni[1];
  c.nck = c.ndim == 3 ? (int)(long long)ni[2] : 1;
  c.dx = gen ? 1.0 : dx[0];
  c.dy = gen ? 1.0 : dx[1];
  c.dz = gen ? 1.0 : (c.ndim == 3 ? dx[2] : dx[0]);
  // src/input.cpp:317-323: an unknown name leaves WENO5
  c.scheme = scheme == "centered4" ? FST_SCHEME_CENTERED4
             : scheme == "quick"   ? FST_SCHEME_QUICK
                                   : FST_SCHEME_WENO5;
  if (gen) {
    if (c.mode == FST_MODE_HYBRID || (c.mode == FST_MODE_MIXED && c.ndim != 3))
      throw DeckError{FST_ERR_UNSUPPORTED,
                      "generalized grids run in the plain FP64 mode (and mixed in 3D)"};
    if (xper || yper || zper)
      throw DeckError{FST_ERR_UNSUPPORTED, "periodic axes are not supported on generalized grids"};
  }
  if (c.ndim == 2 && c.scheme != FST_SCHEME_WENO5 && c.mode != FST_MODE_PLAIN_FP64)
    throw DeckError{FST_ERR_UNSUPPORTED, "fiesta.advection_scheme '" + scheme +
                                             "' runs in the plain FP64 mode"};
  if (c.ng != 3) throw DeckError{FST_ERR_UNSUPPORTED, "fiesta.ng must be 3"};
  d->gen3d = gen && c.ndim == 3;
}

// luaReader::call: fiesta.<f>(a...) must exist and return a number
double call(fst_deck* d, const char* f, double a0, double a1, double a2, double a3) {
  lua_State* L = d->L;
  const int top = lua_gettop(L);
  lua_getglobal(L, "fiesta");
  if (!lua_istable(L, -1)) {  // the deck's own functions may have replaced it
    lua_settop(L, top);
    throw DeckError{FST_ERR_INVALID, "the deck replaced the table 'fiesta'"};
  }
  lua_getfield(L, -1, f);
  if (lua_isnoneornil(L, -1)) {
    lua_settop(L, top);
    throw DeckError{FST_ERR_INVALID,
                    std::string("Could not find fiesta.") + f + " in '" + d->filename + "'"};
  }
  lua_pushnumber(L, a0);
  lua_pushnumber(L, a1);
  lua_pushnumber(L, a2);
  lua_pushnumber(L, a3);
  if (lua_pcall(L, 4, 1, 0) != LUA_OK) {
    const std::string msg = lua_tostring(L, -1) ? lua_tostring(L, -1) : "?";
    lua_settop(L, top);
    throw DeckError{FST_ERR_INVALID, std::string("error running function '") + f + "': " + msg};
  }
  int isnum;
  const double z = lua_tonumberx(L, -1, &isnum);
  lua_settop(L, top);
  if (!isnum)
    throw DeckError{FST_ERR_INVALID, std::string("function '") + f + "' should return a number"};
  return z;
}

void set_error(char* err, size_t errlen, const std::string& msg) {
  if (err && errlen) {
    std::strncpy(err, msg.c_str(), errlen - 1);
    err[errlen - 1] = 0;
  }
}

}  // namespace

extern "C" {

int fst_deck_load(const char* path, fst_deck** out, char* err, size_t errlen) {
  if (!out) return FST_ERR_INVALID;
  *out = nullptr;
  if (!path) {
    set_error(err, errlen, "no deck path");
    return FST_ERR_INVALID;
  }
  fst_deck* d = new fst_deck();
  d->filename = path;
  d->L = luaL_newstate();
  if (!d->L) {
    delete d;
    set_error(err, errlen, "lua state allocation failed");
    return FST_ERR_OOM;
  }
  lua_State* L = d->L;
  lua_newtable(L);
  for (const char* t : kPreset) {
    lua_newtable(L);
    lua_setfield(L, -2, t);
  }
  lua_setglobal(L, "fiesta");
  luaL_openlibs(L);
  if (luaL_loadfile(L, path) || lua_pcall(L, 0, 0, 0)) {
    const std::string msg = std::string("Cannot run config file: ") +
                            (lua_tostring(L, -1) ? lua_tostring(L, -1) : "?");
    lua_close(L);
    delete d;
    set_error(err, errlen, msg);
    return FST_ERR_INVALID;
  }
  lua_getglobal(L, "fiesta");
  const bool ok = lua_istable(L, -1);
  lua_pop(L, 1);
  try {
    if (!ok) throw DeckError{FST_ERR_INVALID, "the deck replaced the table 'fiesta'"};
    read_config(d);
  } catch (const DeckError& e) {
    lua_close(L);
    delete d;
    set_error(err, errlen, e.msg);
    return e.code;
  }
  *out = d;
  return FST_OK;
}

void fst_deck_destroy(fst_deck* d) {
  if (!d) return;
  if (d->L) lua_close(d->L);
  delete d;
}

const char* fst_deck_last_error(const fst_deck* d) { return d ? d->error.c_str() : ""; }

int fst_deck_config(const fst_deck* d, fst_config* cfg) {
  if (!d || !cfg) return FST_ERR_INVALID;
  *cfg = d->cf;
  return FST_OK;
}

int fst_deck_noise(const fst_deck* d, fst_noise_params* np, int* enabled) {
  if (!d || !np || !enabled) return FST_ERR_INVALID;
  // gen3d_func::postStep has no noise filter (src/gen3d.cpp:111-128)
  *enabled = d->noise && !d->gen3d;
  *np = d->np;
  return FST_OK;
}

int fst_deck_grid_nodes(fst_deck* d, const fst_config* c, double* X, size_t n) {
  if (!d || !c || !X) return FST_ERR_INVALID;
  const long long ni = c->nci + 1, nj = c->ncj + 1, nk = c->ndim == 3 ? c->nck + 1 : 1;
  if (n != (size_t)(ni * nj * nk * 3)) return FST_ERR_SIZE;
  std::fill(X, X + n, 0.0);
  try {
    for (int v = 0; v < c->ndim; ++v)
      for (long long k = 0; k < nk; ++k)
        for (long long j = 0; j < nj; ++j)
          for (long long i = 0; i < ni; ++i)
            X[i + ni * (j + nj * (k + nk * v))] =
                call(d, "initialize_grid", (double)i, (double)j, (double)k, (double)v);
  } catch (const DeckError& e) {
    d->error = e.msg;
    return e.code;
  }
  return FST_OK;
}

int fst_deck_initial_conditions(fst_deck* d, const fst_config* c, const double* X, double* U,
                                size_t n) {
  if (!d || !c || !U) return FST_ERR_INVALID;
  const bool gen = c->grid_type == FST_GRID_GENERALIZED;
  if (gen && !X) return FST_ERR_INVALID;
  const int ng = c->ng;
  const long long ngi = c->nci + 2 * ng, ngj = c->ncj + 2 * ng;
  const long long ngk = c->ndim == 3 ? c->nck + 2 * ng : 1;
  const int nv = (c->ndim == 3 ? 4 : 3) + c->ns;
  const int nvt = nv + (c->ceq ? 5 : 0);
  if (n != (size_t)(ngi * ngj * ngk * nvt)) return FST_ERR_SIZE;
  std::fill(U, U + n, 0.0);
  const long long ni = c->nci + 1, nj = c->ncj + 1, nk = c->ndim == 3 ? c->nck + 1 : 1;
  auto node = [&](long long i, long long j, long long k, int v) {
    return X[i + ni * (j + nj * (k + nk * v))];
  };
  const int k0 = c->ndim == 3 ? ng : 0, k1 = c->ndim == 3 ? c->nck + ng : 1;
  try {
    for (int v = 0; v < nv; ++v)
      for (int k = k0; k < k1; ++k)
        for (int j = ng; j < c->ncj + ng; ++j)
          for (int i = ng; i < c->nci + ng; ++i) {
            double x, y, z = 0.0;
            if (!gen) {  // cell centres of a uniform grid (src/input.cpp:462-464)
              x = c->dx * (i - ng) + 0.5 * c->dx;
              y = c->dy * (j - ng) + 0.5 * c->dy;
              if (c->ndim == 3) z = c->dz * (k - ng) + 0.5 * c->dz;
            } else if (c->ndim == 3) {  // the mean of the cell's 8 nodes
              x = y = z = 0.0;
              for (int ix = 0; ix < 2; ++ix)
                for (int iy = 0; iy < 2; ++iy)
                  for (int iz = 0; iz < 2; ++iz) {
                    x += node(i + ix - ng, j + iy - ng, k + iz - ng, 0);
                    y += node(i + ix - ng, j + iy - ng, k + iz - ng, 1);
                    z += node(i + ix - ng, j + iy - ng, k + iz - ng, 2);
                  }
              x = x / 8.0;
              y = y / 8.0;
              z = z / 8.0;
            } else {  // the mean of the cell's 4 nodes
              x = y = 0.0;
              for (int ix = 0; ix < 2; ++ix)
                for (int iy = 0; iy < 2; ++iy) {
                  x += node(i + ix - ng, j + iy - ng, 0, 0);
                  y += node(i + ix - ng, j + iy - ng, 0, 1);
                }
              x = x / 4.0;
              y = y / 4.0;
            }
            U[i + ngi * (j + ngj * ((long long)k + ngk * v))] =
                call(d, "initial_conditions", x, y, z, (double)v);
          }
  } catch (const DeckError& e) {
    d->error = e.msg;
    return e.code;
  }
  return FST_OK;
}

}  // extern "C"
