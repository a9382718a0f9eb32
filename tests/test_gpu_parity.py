"""GPU parity of the plain FP64 path against the oracle and the golden
vectors, through the C ABI.

Bar: IEEE-equal results (every element ==, so only the sign of a zero may
differ) for every golden case, every BC known-answer test, and randomised
configurations; at the benchmark size, size-independent properties.
"""
import numpy as np
import pytest

from fiesta_gb300 import abi
from fiesta_gb300.solver import Solver, initial_conditions
from oracle.oracle import Oracle
from tests import test_oracle as kat
from tests.golden_io import interior, rel_l2, same

pytestmark = pytest.mark.gpu


def test_gpu_golden_vectors(golden_cases):
    for c in golden_cases:
        s = Solver(c.cfg)
        s.set_state(c.U0)
        s.apply_bcs()
        R = s.compute_rhs()
        assert same(R, c.R1), (c.name, np.abs(R - c.R1).max())
        s = Solver(c.cfg)
        s.set_state(c.U0)
        s.rk_step(c.steps)
        U = s.get_state()
        assert same(U, c.UN), (c.name, rel_l2(U, c.UN))
        assert same(s.secondary(), c.SN), c.name


@pytest.mark.parametrize("kat_fn", [kat.outflow_kat, kat.reflective_kat, kat.hydrostatic_kat,
                                    kat.periodic_kat])
def test_gpu_bc_known_answers(kat_fn):
    kat_fn(Solver)


def _random_case(seed, ceq=True, visc=True, big=False):
    rng = np.random.default_rng(seed)
    ndim = 2 + seed % 2
    ns = int(rng.integers(1, 6))
    sp = [dict(gamma=float(rng.uniform(1.2, 1.7)), M=float(rng.uniform(0.5, 3.0)),
               mu=float(rng.uniform(1e-3, 1e-2))) for _ in range(ns)]
    lo, hi = (20, 70) if big else (1, 12)
    n = tuple(int(x) for x in rng.integers(lo, hi, size=3))
    bcs = tuple(rng.choice(["outflow", "reflective", "noslip", "hydrostatic"], size=6))
    per = tuple(bool(x) for x in rng.integers(0, 2, size=3))
    L = tuple(float(x) for x in rng.choice([1.0, 0.7], size=3))
    return abi.make_config(ndim, n, L=L, dt=1e-3, species=sp, R=1.0, visc=visc, ceq=ceq,
                           buoyancy=bool(rng.integers(0, 2)), g=0.3, rho_ref=0.5,
                           periodic=per, bcs=bcs)


@pytest.mark.parametrize("seed", list(range(12)))
def test_gpu_matches_oracle_random(seed):
    cfg = _random_case(seed, ceq=seed % 3 != 0, visc=seed % 4 != 1)
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, seed)
    o, g = Oracle(cfg), Solver(cfg)
    for x in (o, g):
        x.set_state(U0)
        x.apply_bcs()
    assert same(g.get_state(), o.get_state())
    assert same(g.compute_rhs(), o.compute_rhs())
    o.rk_step(3)
    g.rk_step(3)
    assert same(g.get_state(), o.get_state()), rel_l2(g.get_state(), o.get_state())


@pytest.mark.parametrize("seed", [101, 102])
def test_gpu_matches_oracle_medium(seed):
    cfg = _random_case(seed, big=True)
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, seed)
    o, g = Oracle(cfg), Solver(cfg)
    for x in (o, g):
        x.set_state(U0)
    o.rk_step(2)
    g.rk_step(2)
    assert same(g.get_state(), o.get_state())


def mixing_config(n, mode=abi.MODE_PLAIN_FP64, dt=2e-8):
    sp = [dict(gamma=g, M=m / 1000.0, mu=mu) for g, m, mu in
          zip([1.4, 1.67, 1.3, 1.32, 1.4], [28.96, 4.0, 44.0, 16.0, 2.0],
              [1.8e-5, 1.99e-5, 1.47e-5, 1.1e-5, 0.88e-5])]
    return abi.make_config(3, n, dt=dt, species=sp, visc=True, ceq=True, kap=10.0, eps=0.4,
                           alpha=40.0, mode=mode)


def test_gpu_mixing_rhs_matches_oracle_64():
    cfg = mixing_config((64, 64, 64))
    U0 = initial_conditions(cfg, abi.IC_MIXING_3D, 20261206, p_ambient=1e5, T_ambient=300.0,
                            nkernels=8)
    o, g = Oracle(cfg), Solver(cfg)
    for x in (o, g):
        x.set_state(U0)
    assert same(g.compute_rhs(), o.compute_rhs())
    o.rk_step(1)
    g.rk_step(1)
    assert same(g.get_state(), o.get_state())


def test_gpu_full_size_periodic_conservation():
    # 256^3, 5 species: with periodic boundaries the flux-form update
    # conserves every species mass; drift is round-off only.
    cfg = mixing_config((256, 256, 256))
    cfg.xper = cfg.yper = cfg.zper = 1
    U0 = initial_conditions(cfg, abi.IC_MIXING_3D, 20261206, p_ambient=1e5, T_ambient=300.0,
                            nkernels=8)
    g = Solver(cfg)
    g.set_state(U0)
    g.rk_step(2)
    U = g.get_state()
    assert g.check_finite()
    for s in range(5):
        m0 = interior(cfg, U0[..., 4 + s]).sum()
        m1 = interior(cfg, U[..., 4 + s]).sum()
        assert abs(m1 - m0) <= 1e-11 * abs(m0), (s, m0, m1)


@pytest.mark.parametrize("n", [(1, 5, 4), (2, 1, 3), (5, 2, 1)])
def test_gpu_degenerate_periodic(n):
    sp = [dict(gamma=1.4, M=1.0, mu=1e-3), dict(gamma=1.6, M=2.0, mu=2e-3)]
    cfg = abi.make_config(3, n, dt=1e-3, species=sp, R=1.0, visc=True, ceq=True,
                          periodic=(True, True, True))
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, 4)
    o, g = Oracle(cfg), Solver(cfg)
    for x in (o, g):
        x.set_state(U0)
        x.apply_bcs()
    assert same(g.compute_rhs(), o.compute_rhs())
    o.rk_step(2)
    g.rk_step(2)
    assert same(g.get_state(), o.get_state())


def test_gpu_mixed_beyond_32bit_state_indices():
    """530^3 interior, 5 species, C-equation: the state holds 536^3 x 14 =
    2.16e9 doubles, past 2^31, so every variable offset of the last fields
    needs 64-bit indexing.  One mixed-precision step with periodic
    boundaries: finite, species masses conserved to round-off, and the last
    C-variable of the last interior cell updated."""
    cfg = mixing_config((530, 530, 530))
    cfg.mode = abi.MODE_MIXED
    cfg.xper = cfg.yper = cfg.zper = 1
    ngi, ngj, ngk, nvt = abi.dims(cfg)
    assert ngi * ngj * ngk * nvt > 2 ** 31
    ng = cfg.ng
    # a smooth periodic state built by broadcasting (fast at this size)
    tp = 2.0 * np.pi
    x = (np.arange(ngi) - ng + 0.5) / 530
    sx = np.sin(tp * x)[:, None, None]
    cy = np.cos(tp * x)[None, :, None]
    sz = np.sin(tp * x)[None, None, :]
    U0 = np.zeros((ngi, ngj, ngk, nvt), order="F")
    rho = 0.0
    for s_ in range(5):
        U0[..., 4 + s_] = 0.2 * (1.0 + 0.05 * (s_ + 1) * sx * cy)
        rho = rho + U0[..., 4 + s_]
    U0[..., 0] = 10.0 * sz * rho
    U0[..., 3] = 2.5e5 * (1.0 + 0.01 * cy * sz)
    U0[..., nvt - 1] = 0.1  # a C-variable the step must move
    g = Solver(cfg)
    g.set_state(U0)
    g.rk_step(1)
    assert g.check_finite()
    U = g.get_state()
    last = (ngi - ng - 1, ngj - ng - 1, ngk - ng - 1, nvt - 1)
    assert U[last] != U0[last]
    for s in range(5):
        m0 = interior(cfg, U0[..., 4 + s]).sum()
        m1 = interior(cfg, U[..., 4 + s]).sum()
        assert abs(m1 - m0) <= 1e-9 * abs(m0), (s, m0, m1)
