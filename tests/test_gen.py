"""Generalized (curvilinear) grids — the reference's gen2d / gen3d modules —
and the 2D centered4 / QUICK advection schemes.

CPU: the oracle restatement against golden vectors made by the reference's
own sources (tests/golden/make_golden_gen.py), against the reference itself on
random cases where its tree is present, and the configuration checks that
need no GPU.  GPU (marked): the CUDA path against the same golden vectors and
the oracle, bit for bit (IEEE equality; NaN where the reference gives NaN).
"""
import ctypes as C

import numpy as np
import pytest

from fiesta_gb300 import abi
from fiesta_gb300.solver import FstError, Solver, initial_conditions, lib
from oracle.oracle import Oracle, Reference
from tests.golden_io import load_gen, same, wavy_nodes

GEN = abi.GRID_GENERALIZED
UNIT = (1.0, 1.0, 1.0)


@pytest.fixture(scope="module")
def gen_cases():
    cases = load_gen()
    assert len(cases) >= 6
    return cases


def _run(make, c):
    """(metrics, R1, UN) of fixture case c through a checker or the GPU."""
    gen = c.cfg.grid_type == GEN
    x = make(c.cfg)
    x.set_state(c.U0)
    MT = None
    if gen:
        x.set_grid(c.X)
        MT = x.metrics()
    R1 = x.compute_rhs()
    x = make(c.cfg)
    x.set_state(c.U0)
    if gen:
        x.set_grid(c.X)
    x.rk_step(c.steps)
    return MT, R1, x.get_state()


def test_oracle_matches_golden(gen_cases):
    for c in gen_cases:
        MT, R1, UN = _run(Oracle, c)
        if MT is not None:
            assert same(MT, c.MT), c.name
        assert same(R1, c.R1), c.name
        assert same(UN, c.UN), c.name


def _random_gen(seed, ndim):
    rng = np.random.default_rng(seed)
    ns = int(rng.integers(1, 4))
    sp = [dict(gamma=float(rng.uniform(1.2, 1.7)), M=float(rng.uniform(0.5, 3.0)), mu=1e-5)
          for _ in range(ns)]
    n = tuple(int(x) for x in rng.integers(1, 11, size=3))
    scheme = int(rng.integers(1, 4)) if ndim == 2 else 1
    cfg = abi.make_config(ndim, n, dx=UNIT, dt=1e-4, species=sp, R=1.0, grid_type=GEN,
                          scheme=scheme, ceq=bool(rng.integers(0, 2)))
    return cfg, float(rng.uniform(0.0, 0.28))


@pytest.mark.skipif(not Reference.available(), reason="reference checker not built")
@pytest.mark.parametrize("seed", list(range(8)))
def test_oracle_matches_reference_random(seed):
    cfg, amp = _random_gen(seed, 2 + seed % 2)
    X = wavy_nodes(cfg, amp=amp)
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, seed)
    r, o = Reference(cfg), Oracle(cfg)
    for x in (r, o):
        x.set_state(U0)
        x.apply_bcs()
        x.set_grid(X)
    assert same(o.metrics(), r.metrics())
    assert same(o.compute_rhs(), r.compute_rhs())
    o.rk_step(2)
    r.rk_step(2)
    assert same(o.get_state(), r.get_state())


@pytest.mark.skipif(not Reference.available(), reason="reference checker not built")
def test_oracle_matches_reference_zero_ghosts():
    """The modules apply no BCs: with the interior-only initial state that
    loadInitialConditions writes, zero-density ghosts give NaN near the
    boundary in the reference, and the oracle reproduces where."""
    cfg = abi.make_config(2, (9, 8), dx=UNIT, dt=1e-4, species=[dict(gamma=1.4, M=1.0)],
                          R=1.0, grid_type=GEN)
    X = wavy_nodes(cfg, amp=0.2)
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, 5)
    r, o = Reference(cfg), Oracle(cfg)
    for x in (r, o):
        x.set_state(U0)
        x.set_grid(X)
    Rr, Ro = r.compute_rhs(), o.compute_rhs()
    assert np.isnan(Rr).any() and same(Ro, Rr)


def test_config_checks_without_gpu():
    L = lib()
    base = dict(dx=UNIT, dt=1e-4, R=1.0, grid_type=GEN)
    bad = [abi.make_config(3, (4, 4, 4), periodic=(False, True, False), **base),
           abi.make_config(3, (4, 4, 4), mode=abi.MODE_HYBRID, **base),
           abi.make_config(2, (4, 4), mode=abi.MODE_MIXED, **base),
           abi.make_config(2, (4, 4), mode=abi.MODE_MIXED, scheme="quick", dx=UNIT),
           abi.make_config(2, (4, 4), scheme=7, dx=UNIT)]
    for cfg in bad:
        with pytest.raises(FstError):
            Solver(cfg)
    cfg = abi.make_config(3, (4, 5, 6), **base)
    assert L.fst_grid_size(cfg) == 5 * 6 * 7 * 3
    assert L.fst_metrics_size(cfg) == 10 * 11 * 12 * 9
    cfg2 = abi.make_config(2, (4, 5), **base)
    assert L.fst_grid_size(cfg2) == 5 * 6 * 1 * 3
    assert L.fst_metrics_size(cfg2) == 10 * 11 * 4


# --------------------------------------------------------------------- GPU
@pytest.mark.gpu
def test_gpu_matches_golden(gen_cases):
    for c in gen_cases:
        MT, R1, UN = _run(Solver, c)
        if MT is not None:
            assert same(MT, c.MT), c.name
        assert same(R1, c.R1), (c.name, np.nanmax(np.abs(R1 - c.R1)))
        assert same(UN, c.UN), c.name


@pytest.mark.gpu
@pytest.mark.parametrize("seed", list(range(10)))
def test_gpu_matches_oracle_random(seed):
    cfg, amp = _random_gen(100 + seed, 2 + seed % 2)
    X = wavy_nodes(cfg, amp=amp)
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, seed)
    o, g = Oracle(cfg), Solver(cfg)
    for x in (o, g):
        x.set_state(U0)
        x.apply_bcs()
        x.set_grid(X)
    assert same(g.metrics(), o.metrics())
    assert same(g.compute_rhs(), o.compute_rhs())
    o.rk_step(3)
    g.rk_step(3)
    assert same(g.get_state(), o.get_state())


@pytest.mark.gpu
@pytest.mark.parametrize("ndim,n", [(3, (40, 33, 29)), (2, (300, 260, 1))])
def test_gpu_matches_oracle_medium(ndim, n):
    cfg = abi.make_config(ndim, n, dx=UNIT, dt=2e-5,
                          species=[dict(gamma=1.4, M=1.0), dict(gamma=1.6, M=0.4)], R=1.0,
                          grid_type=GEN)
    X = wavy_nodes(cfg, amp=0.25)
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, 9)
    o, g = Oracle(cfg), Solver(cfg)
    for x in (o, g):
        x.set_state(U0)
        x.apply_bcs()
        x.set_grid(X)
    o.rk_step(2)
    g.rk_step(2)
    assert same(g.get_state(), o.get_state())


@pytest.mark.gpu
def test_gpu_zero_ghosts_nan_pattern():
    cfg = abi.make_config(3, (7, 6, 5), dx=UNIT, dt=1e-4, species=[dict(gamma=1.4, M=1.0)],
                          R=1.0, grid_type=GEN)
    X = wavy_nodes(cfg, amp=0.2)
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, 3)
    o, g = Oracle(cfg), Solver(cfg)
    for x in (o, g):
        x.set_state(U0)
        x.set_grid(X)
    Ro, Rg = o.compute_rhs(), g.compute_rhs()
    assert np.isnan(Ro).any() and same(Rg, Ro)


@pytest.mark.gpu
def test_gpu_generalized_call_order_and_limits():
    cfg = abi.make_config(2, (6, 6), dx=UNIT, dt=1e-4, R=1.0, grid_type=GEN)
    g = Solver(cfg)
    with pytest.raises(FstError):
        g.compute_rhs()  # before set_grid
    with pytest.raises(FstError):
        g.rk_step(1)
    with pytest.raises((FstError, ValueError)):
        g.set_grid(np.zeros((3, 3, 1, 3)))
    X = np.asfortranarray(wavy_nodes(cfg))
    rc = lib().fst_set_grid(g._ctx, X.ctypes.data_as(C.POINTER(C.c_double)), X.size - 1)
    assert rc == abi.FST_ERR_SIZE
    g.set_grid(wavy_nodes(cfg))
    g3 = Solver(abi.make_config(3, (4, 4, 4), dx=UNIT, dt=1e-4, R=1.0, grid_type=GEN))
    with pytest.raises(FstError):
        g3.noise_filter(1e-5, 1e-3)  # gen3d_func has no noise filter
    c = Solver(abi.make_config(2, (6, 6)))
    with pytest.raises(FstError):
        c.set_grid(wavy_nodes(cfg))


@pytest.mark.gpu
def test_gpu_deck_to_gen2d_module():
    """A generalized deck through the module mirror (Gen2D): grid from
    fiesta.initialize_grid, cell centres from node averages, metrics at
    preSim, steps without BCs — equal to the oracle on the same inputs."""
    from fiesta_gb300 import deck
    from fiesta_gb300.solver import Gen2D, module_for, rkAdvance
    from tests.test_deck import DECK_GEN2D
    d = deck.load(text=DECK_GEN2D)
    cfg = d.config()
    f = module_for(cfg)(cfg)
    assert isinstance(f, Gen2D)
    f.grid = d.grid_nodes(cfg)
    U0 = d.initial_conditions(cfg, f.grid)
    f.var = U0
    f.preSim()
    o = Oracle(cfg)
    o.set_state(U0)
    o.set_grid(f.grid)
    assert same(f.metrics, o.metrics())
    for _ in range(3):
        rkAdvance(cfg, f)
    o.rk_step(3)
    assert same(f.var, o.get_state())


@pytest.mark.gpu
def test_gpu_gen3d_benchmark_size_matches_oracle():
    """The generalized leg of bench.py at its full size (wavy 256^3 grid,
    5 species): metrics and one step bit for bit with the oracle."""
    import bench
    cfg = bench.gen3d_cfg(256, 1.0)
    U0, X, dt = bench.gen3d_state(cfg, 1.0)
    cfg.dt = dt
    o, g = Oracle(cfg), Solver(cfg)
    for x in (o, g):
        x.set_state(U0)
        x.apply_bcs()
        x.set_grid(X)
    assert same(g.metrics(), o.metrics())
    o.rk_step(1)
    g.rk_step(1)
    assert same(g.get_state(), o.get_state())


@pytest.mark.gpu
def test_gpu_terrain_grid_matches_oracle():
    """A terrain-following grid (readTerrain's nodes from a height field)
    through the generalized 3D path, bit for bit with the oracle."""
    from fiesta_gb300.grids import terrain_nodes
    cfg = abi.make_config(3, (12, 10, 8), dx=UNIT, dt=1e-4, species=[dict(gamma=1.4, M=1.0)],
                          R=1.0, grid_type=GEN)
    i, j = np.meshgrid(np.arange(13), np.arange(11), indexing="ij")
    hgt = 0.1 * np.sin(0.5 * i) * np.cos(0.4 * j)
    X = terrain_nodes(cfg, hgt, 1.0 / 12, 1.0 / 10, 1.0)
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, 8)
    o, g = Oracle(cfg), Solver(cfg)
    for x in (o, g):
        x.set_state(U0)
        x.apply_bcs()
        x.set_grid(X)
    assert same(g.metrics(), o.metrics())
    o.rk_step(2)
    g.rk_step(2)
    assert same(g.get_state(), o.get_state())


def _rel(a, b):
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return d / n if n > 0 else d


@pytest.mark.gpu
@pytest.mark.parametrize("n,ceq", [((24, 20, 18), False), ((40, 33, 29), True)])
def test_gpu_mixed_generalized_within_1e5_of_fp64(n, ceq):
    """The mixed-precision form of the generalized 3D module against its FP64
    form (bit-identical to the reference): every conserved field within
    rel-L2 1e-5 after a few steps (momenta by their increments)."""
    sp = [dict(gamma=1.4, M=0.02896), dict(gamma=1.67, M=0.004)]
    cfg = abi.make_config(3, n, dx=UNIT, dt=1.0, species=sp, grid_type=GEN, ceq=ceq)
    U0 = initial_conditions(cfg, abi.IC_MIXING_3D, 4, p_ambient=1e5, T_ambient=300.0,
                            nkernels=3)
    X = wavy_nodes(cfg, amp=0.25)
    import bench
    S = bench.max_wave_speed(cfg, U0) * n[0]  # cells per second on the unit box
    cfg.dt = 0.4 / S
    mcfg = abi.config_from_dict(abi.config_to_dict(cfg))
    mcfg.mode = abi.MODE_MIXED
    p, m = Solver(cfg), Solver(mcfg)
    for x in (p, m):
        x.set_state(U0)
        x.apply_bcs()
        x.set_grid(X)
    assert same(m.metrics(), p.metrics())
    p.rk_step(4)
    m.rk_step(4)
    Up, Um = p.get_state(), m.get_state()
    ng = cfg.ng
    for v in range(abi.dims(cfg)[3]):
        a = Um[ng:-ng, ng:-ng, ng:-ng, v] - (U0[ng:-ng, ng:-ng, ng:-ng, v] if v < 3 else 0)
        b = Up[ng:-ng, ng:-ng, ng:-ng, v] - (U0[ng:-ng, ng:-ng, ng:-ng, v] if v < 3 else 0)
        assert _rel(a, b) <= 1e-5, (v, _rel(a, b))
