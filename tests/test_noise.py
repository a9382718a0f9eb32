"""The postStep noise filter (src/cart3d.cpp:319-374, src/cart2d.cpp:257-307,
src/noise.hpp): the oracle against the reference's own sources compiled here
(serial loop order, the only order with a defined result), and the library's
fst_noise_filter against the oracle, bit for bit."""
import numpy as np
import pytest

from fiesta_gb300 import abi
from fiesta_gb300.solver import initial_conditions
from oracle.oracle import Oracle, Reference
from tests.golden_io import same

CASES = [  # ndim, cells, ceq, mode, nt, dh, coff
    (3, (9, 8, 7), False, 1, 1, 1e-3, 0.0),
    (3, (10, 7, 6), True, 1, 2, 1e-3, 0.5),
    (3, (8, 8, 8), True, 2, 1, 1e-2, 0.0),
    (3, (19, 17, 10), True, 1, 1, 5e-4, 0.8),
    (2, (20, 17), False, 1, 1, 1e-3, 0.0),
    (2, (19, 22), True, 2, 2, 1e-4, 0.3),
    (2, (37, 33), True, 1, 1, 1e-3, 0.2),
]


def _case(ndim, n, ceq, seed):
    sp = [dict(gamma=1.4, M=1.0, mu=1e-3)]
    cfg = abi.make_config(ndim, n, dt=1e-4, species=sp, R=1.0, ceq=ceq)
    rng = np.random.default_rng(seed)
    U = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, seed)
    U = np.asfortranarray(U * (1 + 0.05 * rng.standard_normal(U.shape)))  # roughness
    if ceq:
        U[..., abi.nv_of(cfg) + 1] = np.abs(rng.standard_normal(U.shape[:3]))
    return cfg, U


@pytest.mark.skipif(not Reference.available(), reason="reference checker not built")
@pytest.mark.parametrize("case", CASES)
def test_oracle_noise_matches_reference(case):
    ndim, n, ceq, mode, nt, dh, coff = case
    cfg, U = _case(ndim, n, ceq, 4)
    o, r = Oracle(cfg), Reference(cfg)
    o.set_state(U)
    r.set_state(U)
    for _ in range(2):  # the indicator persists between calls
        o.noise_filter(dh, 0.1, coff, nt, mode)
        r.noise_filter(dh, 0.1, coff, nt, mode)
        assert same(o.get_state(), r.get_state())
        assert np.array_equal(o.noise(), r.noise())
    assert int(o.noise().sum()) > 0 and not np.array_equal(o.get_state(), U)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_noise_matches_oracle(case):
    from fiesta_gb300.solver import Solver
    ndim, n, ceq, mode, nt, dh, coff = case
    cfg, U = _case(ndim, n, ceq, 5)
    o, s = Oracle(cfg), Solver(cfg)
    o.set_state(U)
    s.set_state(U)
    for _ in range(2):
        o.noise_filter(dh, 0.1, coff, nt, mode)
        s.noise_filter(dh, 0.1, coff, nt, mode)
        assert same(s.get_state(), o.get_state())


GEN2D_CASES = [  # cells, mode, nt, dh (gen2d filters both momenta, no cutoff)
    ((9, 8), 1, 1, 1e-3),
    ((20, 17), 2, 2, 1e-3),
    ((2, 6), 1, 1, 1e-3),   # no lattice point along x: removal only
    ((31, 24), 1, 1, 5e-4),
]


def _gen2d_case(n, seed):
    from tests.golden_io import wavy_nodes
    cfg = abi.make_config(2, n, dx=(1.0, 1.0, 1.0), dt=1e-4, species=[dict(gamma=1.4, M=1.0)],
                          R=1.0, ceq=True, grid_type=abi.GRID_GENERALIZED)
    rng = np.random.default_rng(seed)
    U = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, seed)
    U = np.asfortranarray(U * (1 + 0.05 * rng.standard_normal(U.shape)))
    return cfg, U, wavy_nodes(cfg, amp=0.2)


@pytest.mark.skipif(not Reference.available(), reason="reference checker not built")
@pytest.mark.parametrize("case", GEN2D_CASES)
def test_oracle_gen2d_noise_matches_reference(case):
    n, mode, nt, dh = case
    cfg, U, X = _gen2d_case(n, 6)
    o, r = Oracle(cfg), Reference(cfg)
    for x in (o, r):
        x.set_state(U)
        x.set_grid(X)
    for _ in range(2):
        o.noise_filter(dh, 0.1, 0.5, nt, mode)
        r.noise_filter(dh, 0.1, 0.5, nt, mode)
        assert same(o.get_state(), r.get_state())
        assert np.array_equal(o.noise(), r.noise())
    if min(n) > 2:
        assert int(o.noise().sum()) > 0 and not np.array_equal(o.get_state(), U)


@pytest.mark.gpu
@pytest.mark.parametrize("case", GEN2D_CASES)
def test_gpu_gen2d_noise_matches_oracle(case):
    from fiesta_gb300.solver import Solver
    n, mode, nt, dh = case
    cfg, U, X = _gen2d_case(n, 7)
    o, s = Oracle(cfg), Solver(cfg)
    for x in (o, s):
        x.set_state(U)
        x.set_grid(X)
    for _ in range(2):
        o.noise_filter(dh, 0.1, 0.5, nt, mode)
        s.noise_filter(dh, 0.1, 0.5, nt, mode)
        assert same(s.get_state(), o.get_state())


SPARSE_CASES = [  # ndim, cells, dh, nt, planted: rough in one box, a block of -0 momenta
    (3, (40, 36, 33), 1e-2, 1, None),
    (3, (40, 36, 33), 1e-2, 2, None),
    (2, (70, 50), 3e-2, 1, None),
    (3, (40, 36, 33), 1e-2, 2, "nan"),
    (3, (40, 36, 33), 1e-2, 1, "huge"),
    (2, (70, 50), 3e-2, 2, "nan"),
]


def _sparse_case(ndim, n, seed, planted=None):
    """A smooth state with one rough box (flagged cells in a few tiles only)
    and a block of -0 momenta, where an unflagged update still turns -0 into
    +0: the tiles the removal may skip sit beside ones it may not.  `planted`
    puts a NaN or a near-overflow value in an unflagged region, whose
    non-finite results then spread through the sweep across tiles."""
    sp = [dict(gamma=1.4, M=1.0, mu=1e-3)]
    cfg = abi.make_config(ndim, n, dt=1e-4, species=sp, R=1.0, ceq=False)
    rng = np.random.default_rng(seed)
    U = np.array(initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, seed), order="F")
    ng = 3
    box = tuple(slice(ng + 9, ng + 15) for _ in range(ndim))
    U[box] *= 1 + 0.05 * rng.standard_normal(U[box].shape)
    k = () if ndim == 3 else (0,)  # the 2D state is (ngi, ngj, 1, nvt)
    U[tuple(slice(ng + 16, ng + 32) for _ in range(ndim)) + k + (slice(0, ndim),)] = -0.0
    if planted:
        at = (ng + 34, ng + 2) + ((ng + 20,) if ndim == 3 else k)
        U[at + (1,)] = np.nan if planted == "nan" else 1e305
    return cfg, U


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def _same_bits(a, b):
    """Bit patterns, signed zeros included; NaN matches NaN whatever its payload."""
    nan = np.isnan(a) & np.isnan(b)
    return same(a, b) and np.array_equal(_bits(a)[~nan], _bits(b)[~nan])


@pytest.mark.skipif(not Reference.available(), reason="reference checker not built")
@pytest.mark.parametrize("case", SPARSE_CASES)
def test_oracle_sparse_noise_matches_reference(case):
    ndim, n, dh, nt, planted = case
    cfg, U = _sparse_case(ndim, n, 8, planted)
    o, r = Oracle(cfg), Reference(cfg)
    o.set_state(U)
    r.set_state(U)
    o.noise_filter(dh, 0.1, 0.0, nt, 1)
    r.noise_filter(dh, 0.1, 0.0, nt, 1)
    assert _same_bits(o.get_state(), r.get_state())
    flagged = int(o.noise().sum())
    assert 0 < flagged < o.noise().size // 4
    if planted:  # the sweep carried non-finite values past the planted cell
        assert int((~np.isfinite(o.get_state())).sum()) > 1


@pytest.mark.gpu
@pytest.mark.parametrize("case", SPARSE_CASES)
def test_gpu_sparse_noise_matches_oracle(case):
    from fiesta_gb300.solver import Solver
    ndim, n, dh, nt, planted = case
    cfg, U = _sparse_case(ndim, n, 9, planted)
    o, s = Oracle(cfg), Solver(cfg)
    o.set_state(U)
    s.set_state(U)
    for _ in range(2):
        o.noise_filter(dh, 0.1, 0.0, nt, 1)
        s.noise_filter(dh, 0.1, 0.0, nt, 1)
        assert _same_bits(s.get_state(), o.get_state())
    neg0 = _bits(U) == np.uint64(0x8000000000000000)
    assert (neg0 & (_bits(o.get_state()) == 0)).any()  # some -0 became +0


@pytest.mark.gpu
@pytest.mark.parametrize("ndim", [3, 2])
def test_gpu_module_postStep_runs_the_noise_filter(ndim):
    """Cart3D / Cart2D with fiesta.noise on: preStep, rkAdvance, postStep
    (the filter) per step, against the oracle's step + filter."""
    from fiesta_gb300.solver import Cart2D, Cart3D, rkAdvance
    cfg, U = _case(ndim, (10, 7, 6) if ndim == 3 else (19, 22), True, 11)
    np_ = abi.FstNoiseParams(dh=1e-3, eta=0.1, coff=0.5, nt=1, mode=1)
    f = (Cart3D if ndim == 3 else Cart2D)(cfg, noise=np_)
    f.var = U
    f.preSim()
    o = Oracle(cfg)
    o.set_state(U)
    if ndim == 2:
        o.apply_bcs()  # cart2d_func::preSim
    for _ in range(2):
        f.preStep()
        rkAdvance(cfg, f)
        f.postStep()
        o.rk_step(1)
        o.noise_filter(1e-3, 0.1, 0.5, 1, 1)
    assert same(f.var, o.get_state())


@pytest.mark.gpu
def test_gpu_noise_graph_follows_parameter_changes():
    """The sweeps replay as a captured CUDA graph; a call with other
    parameters (eta, nt, mode, cutoff) must re-capture, and a profiled call
    (kernels launched one by one) must give the same bits."""
    from fiesta_gb300.solver import Solver
    cfg, U = _case(3, (19, 17, 10), True, 12)
    calls = [(1e-3, 0.1, 0.5, 1, 1), (1e-3, 0.1, 0.5, 1, 1), (1e-3, 0.2, 0.5, 1, 1),
             (1e-3, 0.2, 0.5, 2, 1), (5e-4, 0.2, 0.0, 2, 2), (1e-3, 0.1, 0.5, 1, 1)]
    o, s, p = Oracle(cfg), Solver(cfg), Solver(cfg)
    for x in (o, s, p):
        x.set_state(U)
    p.set_profiling(True)
    for args in calls:
        o.noise_filter(*args)
        s.noise_filter(*args)
        p.noise_filter(*args)
        assert _same_bits(s.get_state(), o.get_state()), args
        assert _same_bits(p.get_state(), o.get_state()), args
    assert any(k.startswith("noise_remove") for k in p.kernel_times())
