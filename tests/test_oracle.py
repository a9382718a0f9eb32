"""CPU tests of the oracle (the checker the GPU path is judged against).

1. Golden vectors: the oracle reproduces, bit for bit, the reference's own
   sources run on the same inputs (tests/golden/make_golden.py).
2. The reference's BC known-answer tests (tests/bc_outflow.cpp,
   bc_reflective.cpp, bc_hydrostatic.cpp, test.cpp "Periodic BC Test" of the
   reference), with their exact asserted values.
3. Where the reference tree is present, randomised cross-checks against it.
"""
import numpy as np
import pytest

from fiesta_gb300 import abi
from oracle.oracle import Oracle, Reference
from tests.golden_io import same


def test_golden_rhs_and_steps(golden_cases):
    assert len(golden_cases) >= 6
    for c in golden_cases:
        o = Oracle(c.cfg)
        o.set_state(c.U0)
        o.apply_bcs()
        assert same(o.compute_rhs(), c.R1), c.name
        o = Oracle(c.cfg)
        o.set_state(c.U0)
        o.rk_step(c.steps)
        assert same(o.get_state(), c.UN), c.name
        assert same(o.secondary(), c.SN), c.name


def bc_fixture_config(per=(False, False, False), bcs=("outflow",) * 6, ndim=3, nck=3):
    # tests/common/test.cpp:19-102: 3x3x3 interior, ng=3, nvt=nv=5, dx=1,
    # gamma=1, R=1 (one species); nvt=5 matches ns=1 in 3D without ceq.
    return abi.make_config(ndim, (3, 3, nck), dx=(1.0, 1.0, 1.0), dt=1.0, R=1.0,
                           species=[dict(gamma=1.4, M=1.0, mu=1.0)], periodic=per, bcs=bcs)


def _run_bc(make, cfg, setter):
    o = make(cfg)
    V = np.zeros(o.shape, order="F")
    setter(V)
    o.set_state(V)
    o.apply_bcs()
    return o.get_state()


def outflow_kat(make):
    cfg = bc_fixture_config(bcs=("outflow",) * 6)

    def xy(V):
        for (i, j), val in zip([(3, 3), (4, 3), (5, 3), (3, 4), (4, 4), (5, 4), (3, 5), (4, 5), (5, 5)],
                               range(1, 10)):
            V[i, j, 3, 0] = val
    V = _run_bc(make, cfg, xy)
    # tests/bc_outflow.cpp:48-55
    assert V[4, 0, 3, 0] == 8 and V[0, 4, 3, 0] == 6 and V[4, 8, 3, 0] == 2 and V[8, 4, 3, 0] == 4
    assert V[0, 0, 3, 0] == 9 and V[8, 0, 3, 0] == 7 and V[0, 8, 3, 0] == 3 and V[8, 8, 3, 0] == 1

    def yz(V):
        for (j, k), val in zip([(3, 3), (4, 3), (5, 3), (3, 4), (4, 4), (5, 4), (3, 5), (4, 5), (5, 5)],
                               range(1, 10)):
            V[3, j, k, 0] = val
    V = _run_bc(make, cfg, yz)
    # tests/bc_outflow.cpp:72-79
    assert V[3, 4, 0, 0] == 8 and V[3, 0, 4, 0] == 6 and V[3, 4, 8, 0] == 2 and V[3, 8, 4, 0] == 4
    assert V[3, 0, 0, 0] == 9 and V[3, 8, 0, 0] == 7 and V[3, 0, 8, 0] == 3 and V[3, 8, 8, 0] == 1


def reflective_kat(make):
    cfg = bc_fixture_config(bcs=("reflective",) * 6)

    def xy(V):
        for (i, j), val in zip([(3, 3), (4, 3), (5, 3), (3, 4), (4, 4), (5, 4), (3, 5), (4, 5), (5, 5)],
                               range(1, 10)):
            V[i, j, 3, 0] = val
            V[i, j, 3, 1] = val
    V = _run_bc(make, cfg, xy)
    # tests/bc_reflective.cpp:47-54
    exp = {(4, 0): (8, -8), (0, 4): (-6, 6), (4, 8): (2, -2), (8, 4): (-4, 4),
           (0, 0): (-9, -9), (8, 0): (-7, -7), (0, 8): (-3, -3), (8, 8): (-1, -1)}
    for (i, j), (a, b) in exp.items():
        assert V[i, j, 3, 0] == a and V[i, j, 3, 1] == b, (i, j)

    def yz(V):
        for (j, k), val in zip([(3, 3), (4, 3), (5, 3), (3, 4), (4, 4), (5, 4), (3, 5), (4, 5), (5, 5)],
                               range(1, 10)):
            V[3, j, k, 1] = val
            V[3, j, k, 2] = val
    V = _run_bc(make, cfg, yz)
    # tests/bc_reflective.cpp:72-79 (y-z plane, momenta 1 and 2)
    exp = {(4, 0): (8, -8), (0, 4): (-6, 6), (4, 8): (2, -2), (8, 4): (-4, 4),
           (0, 0): (-9, -9), (8, 0): (-7, -7), (0, 8): (-3, -3), (8, 8): (-1, -1)}
    for (j, k), (a, b) in exp.items():
        assert V[3, j, k, 1] == a and V[3, j, k, 2] == b, (j, k)


def hydrostatic_kat(make):
    cfg = bc_fixture_config(bcs=("outflow", "outflow", "hydrostatic", "hydrostatic", "outflow", "outflow"))

    def setter(V):
        cells = [(3, 3), (4, 3), (5, 3), (3, 4), (4, 4), (5, 4), (3, 5), (4, 5), (5, 5)]
        for (i, j), val in zip(cells, range(1, 10)):
            V[i, j, 4, 0:3] = 0.0
            V[i, j, 4, 3] = val
            V[i, j, 4, 4] = 1.0
    V = _run_bc(make, cfg, setter)
    # tests/bc_hydrostatic.cpp:89-98
    assert V[4, 2, 4, 3] == -1 and V[4, 0, 4, 3] == -7 and V[0, 4, 4, 3] == 6
    assert V[4, 8, 4, 3] == 17 and V[8, 4, 4, 3] == 4
    assert V[0, 0, 4, 3] == -6 and V[8, 0, 4, 3] == -8 and V[0, 8, 4, 3] == 18 and V[8, 8, 4, 3] == 16


def periodic_kat(make):
    # tests/test.cpp:327-450: 3x3x10 interior, periodic in x, y, z
    cfg = bc_fixture_config(per=(True, True, True), bcs=("reflective",) * 6, nck=10)

    def setter(V):
        for k, val in zip(range(3, 13), range(50, 60)):
            V[4, 4, k, 0] = val
    V = _run_bc(make, cfg, setter)
    assert V[4, 4, 0, 0] == 57 and V[4, 4, 1, 0] == 58 and V[4, 4, 2, 0] == 59
    assert V[4, 4, 13, 0] == 50 and V[4, 4, 14, 0] == 51 and V[4, 4, 15, 0] == 52


@pytest.mark.parametrize("kat", [outflow_kat, reflective_kat, hydrostatic_kat, periodic_kat])
def test_bc_known_answers_oracle(kat):
    kat(Oracle)


@pytest.mark.skipif(not Reference.available(), reason="reference checker not built here")
@pytest.mark.parametrize("kat", [outflow_kat, reflective_kat, hydrostatic_kat, periodic_kat])
def test_bc_known_answers_reference(kat):
    kat(Reference)


@pytest.mark.skipif(not Reference.available(), reason="reference checker not built here")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_matches_reference_random(seed):
    from fiesta_gb300.solver import initial_conditions
    rng = np.random.default_rng(seed)
    ndim = 2 + seed % 2
    ns = int(rng.integers(1, 5))
    sp = [dict(gamma=float(rng.uniform(1.2, 1.7)), M=float(rng.uniform(0.5, 3.0)),
               mu=float(rng.uniform(1e-3, 1e-2))) for _ in range(ns)]
    n = tuple(int(x) for x in rng.integers(4, 9, size=3))
    bcs = tuple(rng.choice(["outflow", "reflective", "noslip", "hydrostatic"], size=6))
    per = tuple(bool(x) for x in rng.integers(0, 2, size=3))
    cfg = abi.make_config(ndim, n, dt=1e-3, species=sp, R=1.0, visc=True, ceq=True,
                          buoyancy=bool(seed % 2), g=0.3, rho_ref=0.5, periodic=per, bcs=bcs)
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, seed)
    o, r = Oracle(cfg), Reference(cfg)
    for x in (o, r):
        x.set_state(U0)
        x.apply_bcs()
    assert same(o.compute_rhs(), r.compute_rhs())
    o.rk_step(3)
    r.rk_step(3)
    assert same(o.get_state(), r.get_state())


@pytest.mark.skipif(not Reference.available(), reason="reference checker not built here")
@pytest.mark.parametrize("n", [(1, 5, 4), (2, 1, 3), (5, 2, 1)])
def test_oracle_matches_reference_degenerate_periodic(n):
    # fewer interior cells than ghost layers along a periodic axis: the
    # periodic copy reads ghosts, so results depend on every ghost value
    from fiesta_gb300.solver import initial_conditions
    sp = [dict(gamma=1.4, M=1.0, mu=1e-3), dict(gamma=1.6, M=2.0, mu=2e-3)]
    cfg = abi.make_config(3, n, dt=1e-3, species=sp, R=1.0, visc=True, ceq=True,
                          periodic=(True, True, True))
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, 4)
    o, r = Oracle(cfg), Reference(cfg)
    for x in (o, r):
        x.set_state(U0)
        x.apply_bcs()
    assert same(o.compute_rhs(), r.compute_rhs())
    o.rk_step(2)
    r.rk_step(2)
    assert same(o.get_state(), r.get_state())


@pytest.mark.parametrize("n", [(24, 20, 16), (33, 17, 19)])
def test_numpy_mixing_ic_equals_compiled_generator(n):
    """The numpy restatement of the mixing generator (oracle/ics.py, used by
    the benchmark's reference arm, which loads no product library) gives the
    compiled generator's bits."""
    from fiesta_gb300.solver import initial_conditions
    from oracle.ics import mixing_3d
    sp = [dict(gamma=g, M=m / 1000.0, mu=1e-5) for g, m in
          zip([1.4, 1.67, 1.3, 1.32, 1.4], [28.96, 4.0, 44.0, 16.0, 2.0])]
    cfg = abi.make_config(3, n, species=sp, visc=True, ceq=True)
    kw = dict(p_ambient=1e5, T_ambient=300.0, nkernels=8)
    A = initial_conditions(cfg, abi.IC_MIXING_3D, 20261206, **kw)
    B = mixing_3d(cfg, 20261206, **kw)
    assert A.shape == B.shape and np.array_equal(A.view(np.uint64), B.view(np.uint64))


def test_fma_build_of_the_oracle_differs_only_by_rounding():
    """The FMA-contracted oracle build (the rounding spread tests use as the
    floor for the C-equation fields) agrees with the strict build to
    rounding on a smooth case."""
    from fiesta_gb300.solver import initial_conditions
    from oracle.oracle import OracleFMA
    cfg = abi.make_config(3, (12, 10, 8), dt=1e-4, species=[dict(gamma=1.4, M=1.0, mu=1e-3)],
                          R=1.0, visc=True, ceq=True)
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, 2)
    a, b = Oracle(cfg), OracleFMA(cfg)
    for x in (a, b):
        x.set_state(U0)
        x.rk_step(2)
    Ua, Ub = a.get_state(), b.get_state()
    assert np.allclose(Ua, Ub, rtol=1e-12, atol=0)
