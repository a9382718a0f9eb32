// fst_host.cpp — host-only parts of libfst: config helpers and the seeded
// initial-condition generator.
//
// The reference fills the initial state by calling the deck's Lua function
// fiesta.initial_conditions(x, y, z, v) once per interior cell and variable
// (loadInitialConditions, src/input.cpp:445-518).  At 256^3-384^3 that is
// 1e8-1e9 Lua calls, so large runs use this compiled generator instead.  It
// uses the reference's cell-centre formula x = dx*(i-ng) + 0.5*dx
// (src/input.cpp:462-464), a splitmix64 stream for every random draw, and no
// libm calls (exp and cos are evaluated here with fixed polynomials), so the
// same seed gives the same bits on x86 and aarch64 when compiled with
// -ffp-contract=off.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/fst.h"

namespace {

struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // uniform in [0, 1) with 53 random bits
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
};

// exp(x) by exponent split and a degree-13 Taylor polynomial on
// |r| <= ln2/2; relative error ~1e-16, bit-reproducible.
double det_exp(double x) {
  if (x < -700.0) return 0.0;
  if (x > 700.0) x = 700.0;
  const double ln2_hi = 0.693147180369123816490;  // high bits of ln 2
  const double ln2_lo = 1.90821492927058770002e-10;
  double kf = std::floor(x * 1.44269504088896338700 + 0.5);
  double r = (x - kf * ln2_hi) - kf * ln2_lo;
  double p = 1.0;
  for (int n = 13; n >= 1; --n) p = 1.0 + p * r / (double)n;
  return std::ldexp(p, (int)kf);
}

// cos(x) by reduction to [-pi, pi] and a degree-24 Taylor polynomial.
double det_cos(double x) {
  const double two_pi = 6.28318530717958647692;
  x = x - two_pi * std::floor(x / two_pi + 0.5);
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int n = 1; n <= 12; ++n) {
    term = -term * x2 / (double)((2 * n - 1) * (2 * n));
    sum = sum + term;
  }
  return sum;
}

struct Grid {
  int ndim, ng, nci, ncj, nck, ngi, ngj, ngk, ns, nv, nvt;
  double dx, dy, dz;
  explicit Grid(const fst_config* c) {
    ndim = c->ndim;
    ng = c->ng;
    nci = c->nci;
    ncj = c->ncj;
    nck = ndim == 3 ? c->nck : 1;
    ngi = nci + 2 * ng;
    ngj = ncj + 2 * ng;
    ngk = ndim == 3 ? nck + 2 * ng : 1;
    ns = c->ns;
    nv = (ndim == 3 ? 4 : 3) + ns;
    nvt = nv + (c->ceq ? 5 : 0);
    dx = c->dx;
    dy = c->dy;
    dz = ndim == 3 ? c->dz : c->dx;
  }
  size_t cells() const { return (size_t)ngi * ngj * ngk; }
  size_t at(int i, int j, int k, int v) const {
    return (size_t)i + (size_t)ngi * ((size_t)j + (size_t)ngj * ((size_t)k + (size_t)ngk * v));
  }
};

// Writes one cell from primitive values: partial densities rho_s, velocity,
// pressure.  Energy uses the mixture EOS of calculateRhoPT
// (src/secondary.hpp:109-151): E = p/(gamma_mix-1) + 0.5*rho*|u|^2.
void put_cell(const fst_config* c, const Grid& g, double* U, int i, int j, int k,
              const double* rho_s, const double* u, double p) {
  double rho = 0.0, Cp = 0.0, Cv = 0.0;
  for (int s = 0; s < g.ns; ++s) rho = rho + rho_s[s];
  for (int s = 0; s < g.ns; ++s) {
    double Rs = c->R / c->M[s], gs = c->gamma[s];
    double Y = rho_s[s] / rho;
    Cp = Cp + Y * (gs * Rs / (gs - 1.0));
    Cv = Cv + Y * (Rs / (gs - 1.0));
  }
  double gam = Cp / Cv;
  double ke = 0.0;
  for (int d = 0; d < g.ndim; ++d) ke = ke + u[d] * u[d];
  ke = 0.5 * rho * ke;
  for (int d = 0; d < g.ndim; ++d) U[g.at(i, j, k, d)] = rho * u[d];
  U[g.at(i, j, k, g.ndim)] = p / (gam - 1.0) + ke;
  for (int s = 0; s < g.ns; ++s) U[g.at(i, j, k, g.ndim + 1 + s)] = rho_s[s];
}

double mix_R(const fst_config* c, const double* Y, int ns) {
  double r = 0.0;
  for (int s = 0; s < ns; ++s) r = r + Y[s] * (c->R / c->M[s]);
  return r;
}

// Run f(kb, ke) over [k0, k1) split into contiguous plane ranges, one per
// hardware thread (a few planes or a small grid: the calling thread alone).
template <class F>
void parallel_planes(int k0, int k1, const F& f) {
  const int n = k1 - k0;
  int nt = (int)std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  if (nt > n) nt = n;
  if (nt <= 1 || n < 8) {
    f(k0, k1);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t) {
    const int kb = k0 + (int)((long long)n * t / nt), ke = k0 + (int)((long long)n * (t + 1) / nt);
    th.emplace_back([&f, kb, ke] { f(kb, ke); });
  }
  for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

void fst_config_defaults(fst_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->abi_version = FST_ABI_VERSION;
  c->ndim = 3;
  c->nci = c->ncj = c->nck = 1;
  c->ng = 3;
  c->dx = c->dy = c->dz = 1.0;
  c->ns = 1;
  c->R = 8.314462;  // src/input.cpp:162
  c->gamma[0] = 1.4;
  c->M[0] = 0.02896;
  c->mu[0] = 1.8e-5;
  c->kap = 1.23456;  // src/input.cpp:262 default
  c->g_accel = 9.81;  // src/input.cpp:256 default
  c->mode = FST_MODE_PLAIN_FP64;
}

int fst_nvt(const fst_config* c) {
  int nv = (c->ndim == 3 ? 4 : 3) + c->ns;
  return nv + (c->ceq ? 5 : 0);
}

size_t fst_state_size(const fst_config* c) {
  Grid g(c);
  return g.cells() * (size_t)g.nvt;
}

size_t fst_grid_size(const fst_config* c) {
  const size_t nk = c->ndim == 3 ? (size_t)c->nck + 1 : 1;
  return ((size_t)c->nci + 1) * ((size_t)c->ncj + 1) * nk * 3;
}

size_t fst_metrics_size(const fst_config* c) {
  Grid g(c);
  return g.cells() * (size_t)(c->ndim == 3 ? 9 : 4);
}

int fst_fill_initial_conditions(const fst_config* c, const fst_ic_params* ic, double* U,
                                size_t n) {
  if (!c || !ic || !U) return FST_ERR_INVALID;
  if (c->ns < 1 || c->ns > FST_MAX_SPECIES) return FST_ERR_INVALID;
  Grid g(c);
  if (n != g.cells() * (size_t)g.nvt) return FST_ERR_SIZE;
  std::memset(U, 0, n * sizeof(double));
  SplitMix64 rng(ic->seed);
  const int ns = g.ns;
  const double Lx = g.nci * g.dx, Ly = g.ncj * g.dy, Lz = g.nck * g.dz;
  double rho_s[FST_MAX_SPECIES], u[3] = {0, 0, 0};
  auto cx = [&](int i) { return g.dx * (i - g.ng) + 0.5 * g.dx; };
  auto cy = [&](int j) { return g.dy * (j - g.ng) + 0.5 * g.dy; };
  auto cz = [&](int k) { return g.dz * (k - g.ng) + 0.5 * g.dz; };
  const int k0 = g.ndim == 3 ? g.ng : 0, k1 = g.ndim == 3 ? g.ng + g.nck : 1;

  switch (ic->kind) {
    case FST_IC_SHOCK_TUBE_2D: {
      // Sod: left rho=1, p=1; right rho=0.125, p=0.1; diaphragm at x=Lx/2;
      // all mass in species 0.
      for (int k = k0; k < k1; ++k)
        for (int j = g.ng; j < g.ng + g.ncj; ++j)
          for (int i = g.ng; i < g.ng + g.nci; ++i) {
            bool left = cx(i) < 0.5 * Lx;
            for (int s = 0; s < ns; ++s) rho_s[s] = 0.0;
            rho_s[0] = left ? 1.0 : 0.125;
            put_cell(c, g, U, i, j, k, rho_s, u, left ? 1.0 : 0.1);
          }
      break;
    }
    case FST_IC_EXPANSION_3D: {
      // Sphere of species 1 at p_high inside species-0 ambient at p_ambient,
      // both at T_ambient; rho_s = p M_s / (R T); density noise
      // rho *= 1 + noise*(2u-1), one draw per cell in i-fastest order.
      if (ns < 2) return FST_ERR_INVALID;
      const double T0 = ic->T_ambient > 0 ? ic->T_ambient : 300.0;
      const double pa = ic->p_ambient > 0 ? ic->p_ambient : 1e5;
      const double ph = ic->p_high > 0 ? ic->p_high : 1e7;
      const double r0 = ic->radius > 0 ? ic->radius : 0.1;
      for (int k = k0; k < k1; ++k)
        for (int j = g.ng; j < g.ng + g.ncj; ++j)
          for (int i = g.ng; i < g.ng + g.nci; ++i) {
            double x = cx(i) - 0.5 * Lx, y = cy(j) - 0.5 * Ly;
            double z = g.ndim == 3 ? cz(k) - 0.5 * Lz : 0.0;
            bool in = x * x + y * y + z * z < r0 * r0;
            int sp = in ? 1 : 0;
            double p = in ? ph : pa;
            double f = 1.0 + ic->noise * (2.0 * rng.uniform() - 1.0);
            for (int s = 0; s < ns; ++s) rho_s[s] = 0.0;
            rho_s[sp] = p * c->M[sp] / (c->R * T0) * f;
            put_cell(c, g, U, i, j, k, rho_s, u, p);
          }
      break;
    }
    case FST_IC_MIXING_3D: {
      // nkernels Gaussian pressure kernels (amplitude 10-100x ambient, width
      // 0.02-0.08 of the domain, uniform centres) and, per species s >= 1,
      // three Gaussian mass-fraction blobs over a 0.05 floor; Y normalised to
      // sum 1; rho = p / (R_mix T).
      const double T0 = ic->T_ambient > 0 ? ic->T_ambient : 300.0;
      const double pa = ic->p_ambient > 0 ? ic->p_ambient : 1e5;
      const int nk = ic->nkernels > 0 ? ic->nkernels : 8;
      const double L = Lx;
      std::vector<double> kc(nk * 3), ka(nk), kw(nk);
      for (int q = 0; q < nk; ++q) {
        kc[3 * q + 0] = rng.uniform() * Lx;
        kc[3 * q + 1] = rng.uniform() * Ly;
        kc[3 * q + 2] = rng.uniform() * Lz;
        ka[q] = rng.uniform(10.0, 100.0);
        kw[q] = rng.uniform(0.02, 0.08) * L;
      }
      const int nb = 3;
      std::vector<double> bc(ns * nb * 3), ba(ns * nb), bw(ns * nb);
      for (int s = 0; s < ns * nb; ++s) {
        bc[3 * s + 0] = rng.uniform() * Lx;
        bc[3 * s + 1] = rng.uniform() * Ly;
        bc[3 * s + 2] = rng.uniform() * Lz;
        ba[s] = rng.uniform(0.5, 1.0);
        bw[s] = rng.uniform(0.05, 0.15) * L;
      }
      // planes in parallel: every cell's value depends on its position and the
      // draws above only, so the bits do not depend on the thread count
      auto planes = [&](int kb, int ke) {
        double Y[FST_MAX_SPECIES], rho_s[FST_MAX_SPECIES], u[3] = {0, 0, 0};
        for (int k = kb; k < ke; ++k)
        for (int j = g.ng; j < g.ng + g.ncj; ++j)
          for (int i = g.ng; i < g.ng + g.nci; ++i) {
            double x = cx(i), y = cy(j), z = g.ndim == 3 ? cz(k) : 0.0;
            double amp = 0.0;
            for (int q = 0; q < nk; ++q) {
              double ddx = x - kc[3 * q], ddy = y - kc[3 * q + 1], ddz = z - kc[3 * q + 2];
              double r2 = ddx * ddx + ddy * ddy + ddz * ddz;
              amp = amp + ka[q] * det_exp(-r2 / (2.0 * kw[q] * kw[q]));
            }
            double p = pa * (1.0 + amp);
            double tot = 0.0;
            for (int s = 0; s < ns; ++s) {
              double raw = s == 0 ? 1.0 : 0.05;
              if (s > 0)
                for (int b = 0; b < nb; ++b) {
                  int q = s * nb + b;
                  double ddx = x - bc[3 * q], ddy = y - bc[3 * q + 1], ddz = z - bc[3 * q + 2];
                  double r2 = ddx * ddx + ddy * ddy + ddz * ddz;
                  raw = raw + ba[q] * det_exp(-r2 / (2.0 * bw[q] * bw[q])) * 4.0;
                }
              Y[s] = raw;
              tot = tot + raw;
            }
            for (int s = 0; s < ns; ++s) Y[s] = Y[s] / tot;
            double rho = p / (mix_R(c, Y, ns) * T0);
            for (int s = 0; s < ns; ++s) rho_s[s] = Y[s] * rho;
            put_cell(c, g, U, i, j, k, rho_s, u, p);
          }
      };
      parallel_planes(k0, k1, planes);
      break;
    }
    case FST_IC_RT_2D: {
      // Heavy fluid (mostly species 0) over light fluid (mostly species 1), interface at
      // y = Ly/2 + sum_m a_m cos(2 pi m x / Lx + phi_m), sum |a_m| = 0.01 Lx;
      // hydrostatic pressure as in samples/rt2d/fiesta.lua of the reference.
      if (ns < 2) return FST_ERR_INVALID;
      const double rH = ic->rho_heavy > 0 ? ic->rho_heavy : 2.0;
      const double rL = ic->rho_light > 0 ? ic->rho_light : 1.0;
      const double P0 = ic->p_ambient > 0 ? ic->p_ambient : 2.4;
      const double gacc = c->g_accel;
      double am[8], ph[8], asum = 0.0;
      for (int m = 0; m < 8; ++m) {
        am[m] = rng.uniform(-1.0, 1.0);
        ph[m] = rng.uniform(0.0, 6.28318530717958647692);
        asum = asum + std::fabs(am[m]);
      }
      for (int m = 0; m < 8; ++m) am[m] = am[m] / asum * 0.01 * Lx;
      for (int k = k0; k < k1; ++k)
        for (int j = g.ng; j < g.ng + g.ncj; ++j)
          for (int i = g.ng; i < g.ng + g.nci; ++i) {
            double x = cx(i), y = cy(j);
            double h = 0.5 * Ly;
            for (int m = 0; m < 8; ++m)
              h = h + am[m] * det_cos(6.28318530717958647692 * (m + 1) * x / Lx + ph[m]);
            for (int s = 0; s < ns; ++s) rho_s[s] = 0.0;
            double p;
            // each fluid carries 1% of the other species: the hydrostatic
            // ghost fill divides by the first species' density
            // (src/bc.cpp:97, rdx = ndim+1), which must not vanish
            if (y > h) {
              rho_s[0] = 0.99 * rH;
              rho_s[1] = 0.01 * rH;
              p = P0 + rH * gacc * (Ly - y);
            } else {
              rho_s[0] = 0.01 * rL;
              rho_s[1] = 0.99 * rL;
              p = P0 + rL * gacc * (h - y) + rH * gacc * (Ly - h);
            }
            put_cell(c, g, U, i, j, k, rho_s, u, p);
          }
      break;
    }
    case FST_IC_RANDOM_SMOOTH: {
      // Smooth random fields with O(1) values for unit tests: positive
      // partial densities, O(0.3) velocities, positive pressure, and (with
      // the C-equation) positive C variables.
      double ph[16];
      for (int q = 0; q < 16; ++q) ph[q] = rng.uniform(0.0, 6.28318530717958647692);
      double sw[FST_MAX_SPECIES];
      for (int s = 0; s < ns; ++s) sw[s] = rng.uniform(0.3, 1.0);
      for (int k = k0; k < k1; ++k)
        for (int j = g.ng; j < g.ng + g.ncj; ++j)
          for (int i = g.ng; i < g.ng + g.nci; ++i) {
            double x = cx(i) / Lx, y = cy(j) / Ly, z = g.ndim == 3 ? cz(k) / Lz : 0.0;
            double base = 1.0 + 0.3 * det_cos(6.0 * x + ph[0]) * det_cos(5.0 * y + ph[1]) +
                          0.2 * det_cos(4.0 * z + x + ph[2]);
            for (int s = 0; s < ns; ++s)
              rho_s[s] = base * sw[s] * (1.0 + 0.1 * det_cos(3.0 * (s + 1) * x + 2.0 * y - z + ph[3 + s % 8]));
            for (int d = 0; d < g.ndim; ++d)
              u[d] = 0.3 * det_cos(3.0 * x + 2.0 * d + ph[11]) * det_cos(2.0 * y - d + ph[12]) *
                     det_cos(z + d + ph[13]) + 0.05 * (2.0 * rng.uniform() - 1.0);
            double p = 1.0 + 0.5 * det_cos(7.0 * x * y + z + ph[14]) + 0.02 * rng.uniform();
            put_cell(c, g, U, i, j, k, rho_s, u, p);
            if (c->ceq) {
              for (int q = 0; q < 5; ++q)
                U[g.at(i, j, k, g.nv + q)] = 0.1 * (q + 1) * (0.5 + 0.5 * det_cos(4.0 * x + 3.0 * y + q + ph[15]));
            }
            u[0] = u[1] = u[2] = 0.0;
          }
      break;
    }
    default:
      return FST_ERR_INVALID;
  }
  return FST_OK;
}

}  // extern "C"
