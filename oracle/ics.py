"""Seeded initial state of the 3D five-species mixing workload, in numpy.

TEST INFRASTRUCTURE ONLY — used by bench.py's reference arm, which times the
reference's own CPU build and must not load the product library.  It
restates, operation for operation, the FST_IC_MIXING_3D branch of the
product's compiled generator (fst_fill_initial_conditions) so that the
reference arm steps the same bits the GPU arm steps (tests/test_oracle.py
checks the two bit for bit):

* splitmix64 draws, uniform in [0, 1) from the top 53 bits;
* exp by exponent split and a degree-13 Taylor polynomial (no libm);
* nkernels Gaussian pressure kernels (amplitude 10-100x ambient, width
  0.02-0.08 of the domain), per species s >= 1 three Gaussian mass-fraction
  blobs over a 0.05 floor, Y normalised to sum 1, rho = p / (R_mix T);
* cell centres x = dx*(i-ng) + dx/2 (the reference's loadInitialConditions,
  src/input.cpp:462-464); total energy from the mixture EOS of
  calculateRhoPT (src/secondary.hpp:109-151) at rest.
"""
import numpy as np

_M64 = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed):
        self.s = seed & _M64

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & _M64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def uniform(self, a=None, b=None):
        u = float(self.next() >> 11) * (1.0 / 9007199254740992.0)
        return u if a is None else a + (b - a) * u


def det_exp(x):
    """exp(x) elementwise: x = k ln2 + r, Taylor polynomial of degree 13."""
    x = np.asarray(x, dtype=np.float64)
    out_zero = x < -700.0
    x = np.minimum(x, 700.0)
    ln2_hi = 0.693147180369123816490
    ln2_lo = 1.90821492927058770002e-10
    kf = np.floor(x * 1.44269504088896338700 + 0.5)
    r = (x - kf * ln2_hi) - kf * ln2_lo
    p = np.ones_like(x)
    for n in range(13, 0, -1):
        p = 1.0 + p * r / float(n)
    out = np.ldexp(p, kf.astype(np.int64))
    out[out_zero] = 0.0
    return out


def mixing_3d(cfg, seed, p_ambient=1e5, T_ambient=300.0, nkernels=8):
    """State (ngi, ngj, ngk, nvt), Fortran order, for a 3D config."""
    ng, ns = cfg.ng, cfg.ns
    nci, ncj, nck = cfg.nci, cfg.ncj, cfg.nck
    dx, dy, dz = cfg.dx, cfg.dy, cfg.dz
    nv = 4 + ns
    nvt = nv + (5 if cfg.ceq else 0)
    U = np.zeros((nci + 2 * ng, ncj + 2 * ng, nck + 2 * ng, nvt), order="F")
    rng = SplitMix64(seed)
    T0 = T_ambient if T_ambient > 0 else 300.0
    pa = p_ambient if p_ambient > 0 else 1e5
    nk = nkernels if nkernels > 0 else 8
    Lx, Ly, Lz = nci * dx, ncj * dy, nck * dz
    kc, ka, kw = [], [], []
    for _ in range(nk):
        kc.append((rng.uniform() * Lx, rng.uniform() * Ly, rng.uniform() * Lz))
        ka.append(rng.uniform(10.0, 100.0))
        kw.append(rng.uniform(0.02, 0.08) * Lx)
    nb = 3
    bc, ba, bw = [], [], []
    for _ in range(ns * nb):
        bc.append((rng.uniform() * Lx, rng.uniform() * Ly, rng.uniform() * Lz))
        ba.append(rng.uniform(0.5, 1.0))
        bw.append(rng.uniform(0.05, 0.15) * Lx)
    x = (dx * np.arange(nci) + 0.5 * dx)[:, None, None]
    y = (dy * np.arange(ncj) + 0.5 * dy)[None, :, None]
    z = (dz * np.arange(nck) + 0.5 * dz)[None, None, :]
    shape = (nci, ncj, nck)

    def r2(c):
        ddx, ddy, ddz = x - c[0], y - c[1], z - c[2]
        return (ddx * ddx + ddy * ddy) + ddz * ddz

    amp = np.zeros(shape)
    for q in range(nk):
        amp = amp + ka[q] * det_exp(-r2(kc[q]) / (2.0 * kw[q] * kw[q]))
    p = pa * (1.0 + amp)
    Y = []
    tot = np.zeros(shape)
    for s in range(ns):
        raw = np.full(shape, 1.0 if s == 0 else 0.05)
        if s > 0:
            for b in range(nb):
                q = s * nb + b
                raw = raw + ba[q] * det_exp(-r2(bc[q]) / (2.0 * bw[q] * bw[q])) * 4.0
        Y.append(raw)
        tot = tot + raw
    Y = [Ys / tot for Ys in Y]
    Rs = [cfg.R / cfg.M[s] for s in range(ns)]
    rmix = np.zeros(shape)
    for s in range(ns):
        rmix = rmix + Y[s] * Rs[s]
    rho = p / (rmix * T0)
    rho_s = [Y[s] * rho for s in range(ns)]
    # the generator's put_cell: mixture EOS at rest
    rsum = np.zeros(shape)
    for s in range(ns):
        rsum = rsum + rho_s[s]
    Cp = np.zeros(shape)
    Cv = np.zeros(shape)
    for s in range(ns):
        gs = cfg.gamma[s]
        Ys = rho_s[s] / rsum
        Cp = Cp + Ys * (gs * Rs[s] / (gs - 1.0))
        Cv = Cv + Ys * (Rs[s] / (gs - 1.0))
    gam = Cp / Cv
    I = (slice(ng, ng + nci), slice(ng, ng + ncj), slice(ng, ng + nck))
    for d in range(3):
        U[I + (d,)] = rsum * 0.0
    U[I + (3,)] = p / (gam - 1.0) + 0.5 * rsum * 0.0
    for s in range(ns):
        U[I + (4 + s,)] = rho_s[s]
    return U
