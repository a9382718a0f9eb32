"""Accuracy of the mixed-precision path (FP32 fluxes / viscous / C-equation,
FP64 state, FP32-pair equation of state and RK combine) against the FP64
oracle, every state field held to the bar of tests/accuracy.py: 1e-5, or 10x
the field's own condition spread where the reference itself is that
sensitive.
"""
import numpy as np
import pytest

from fiesta_gb300 import abi
from fiesta_gb300.solver import Solver, initial_conditions
from oracle.oracle import Oracle
from tests.accuracy import check_fields, run_pair
from tests.golden_io import interior, rel_l2

pytestmark = pytest.mark.gpu

SP5 = [dict(gamma=g, M=m / 1000.0, mu=mu) for g, m, mu in
       zip([1.4, 1.67, 1.3, 1.32, 1.4], [28.96, 4.0, 44.0, 16.0, 2.0],
           [1.8e-5, 1.99e-5, 1.47e-5, 1.1e-5, 0.88e-5])]


def mixing(n, dt, mode=abi.MODE_MIXED):
    return abi.make_config(3, n, dt=dt, species=SP5, visc=True, ceq=True, kap=10.0, eps=0.4,
                           alpha=40.0, mode=mode)


def test_mixed_mixing_3d_vs_oracle():
    cfg = mixing((48, 40, 32), dt=2e-7)
    U0 = initial_conditions(cfg, abi.IC_MIXING_3D, 20261206, p_ambient=1e5, T_ambient=300.0,
                            nkernels=8)
    check_fields(cfg, *run_pair(cfg, U0, 10), U0)


def test_mixed_expansion_3d_vs_oracle():
    cfg = abi.make_config(3, (32, 32, 32), dt=1e-6, species=SP5[:2], visc=True, ceq=True,
                          mode=abi.MODE_MIXED)
    U0 = initial_conditions(cfg, abi.IC_EXPANSION_3D, 20261204, p_ambient=1e5, T_ambient=300.0,
                            p_high=1e7, radius=0.1 * 32 / 32, noise=0.01)
    check_fields(cfg, *run_pair(cfg, U0, 10), U0)


@pytest.mark.parametrize("case", ["sod", "rt"])
def test_mixed_2d_vs_oracle(case):
    if case == "sod":
        cfg = abi.make_config(2, (100, 40), dt=1e-4, species=[dict(gamma=1.4, M=1.0, mu=0.0)],
                              R=1.0, ceq=True, bcs=("outflow", "outflow", "reflective",
                                                    "reflective", "outflow", "outflow"),
                              mode=abi.MODE_MIXED)
        U0 = initial_conditions(cfg, abi.IC_SHOCK_TUBE_2D, 1)
    else:
        cfg = abi.make_config(2, (48, 96), L=(1.0 / 3.0, 1.0), dt=1e-4,
                              species=[dict(gamma=1.4, M=1.0, mu=0.0), dict(gamma=1.4, M=2.0, mu=0.0)],
                              R=1.0, visc=True, ceq=True, buoyancy=True, g=0.5, rho_ref=1.5,
                              periodic=(True, False, False),
                              bcs=("outflow", "outflow", "hydrostatic", "hydrostatic", "outflow",
                                   "outflow"), mode=abi.MODE_MIXED)
        U0 = initial_conditions(cfg, abi.IC_RT_2D, 7, rho_heavy=2.0, rho_light=1.0, p_ambient=2.4)
    check_fields(cfg, *run_pair(cfg, U0, 50), U0)


def test_mixed_rhs_close_to_oracle():
    cfg = mixing((24, 20, 16), dt=2e-7)
    U0 = initial_conditions(cfg, abi.IC_MIXING_3D, 5, p_ambient=1e5, T_ambient=300.0, nkernels=8)
    m = Solver(cfg)
    m.set_state(U0)
    R = m.compute_rhs()
    cref = abi.config_from_dict(abi.config_to_dict(cfg))
    cref.mode = abi.MODE_PLAIN_FP64
    o = Oracle(cref)
    o.set_state(U0)
    Ro = o.compute_rhs()
    # one RHS evaluation: FP32 face terms (the increments' relative error),
    # FP32-pair switches of the C-equation sources
    for v in range(abi.dims(cfg)[3]):
        e = rel_l2(interior(cfg, R[..., v]), interior(cfg, Ro[..., v]))
        assert e <= 1e-3, (v, e)


def test_mixed_many_species_fallback():
    # 7 species takes the generic (predicated) kernel instance
    sp = [dict(gamma=1.3 + 0.05 * s, M=0.5 + 0.3 * s, mu=1e-3) for s in range(7)]
    cfg = abi.make_config(3, (12, 10, 9), dt=1e-4, species=sp, R=1.0, visc=True, ceq=True,
                          mode=abi.MODE_MIXED)
    U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, 3)
    check_fields(cfg, *run_pair(cfg, U0, 5), U0)


@pytest.mark.parametrize("ns,visc,ceq,buoy", [(1, False, False, False), (3, True, False, True),
                                             (2, False, True, True), (5, True, True, False)])
def test_mixed_3d_term_combinations_ragged_tiles(ns, visc, ceq, buoy):
    """Each optional term on and off, ragged tile edges in x, y and z (the
    3D kernels cover 31x7 columns x 16 planes per block), periodic and
    hydrostatic boundaries."""
    sp = SP5[:ns]
    cfg = abi.make_config(3, (33, 17, 19), dt=1e-7, species=sp, visc=visc, ceq=ceq,
                          buoyancy=buoy, g=9.81, rho_ref=1.0, periodic=(False, True, False),
                          bcs=("outflow", "reflective", "outflow", "outflow", "hydrostatic",
                               "reflective"),
                          mode=abi.MODE_MIXED)
    U0 = initial_conditions(cfg, abi.IC_MIXING_3D, 11 + ns, p_ambient=1e5, T_ambient=300.0,
                            nkernels=4)
    check_fields(cfg, *run_pair(cfg, U0, 6), U0)


@pytest.mark.parametrize("case", ["3d", "2d", "gen3d", "hybrid3d"])
def test_gpu_nan_canary_never_reaches_outputs(case, monkeypatch):
    """FST_DEBUG_CANARY=1 starts the primitive arrays as NaN: entries no
    kernel writes (row padding of the TMA layout, halo beyond the grid) must
    not reach the state, so two steps equal a normal run bit for bit."""
    from tests.golden_io import wavy_nodes
    sp = [dict(gamma=1.4, M=0.02896, mu=1.8e-5), dict(gamma=1.67, M=0.004, mu=1.99e-5)]
    X = None
    if case == "2d":
        cfg = abi.make_config(2, (37, 29), dt=1e-4, species=[dict(gamma=1.4, M=1.0, mu=1e-3)],
                              R=1.0, visc=True, ceq=True, mode=abi.MODE_MIXED)
        U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, 3)
    elif case == "gen3d":
        cfg = abi.make_config(3, (21, 18, 13), dx=(1.0, 1.0, 1.0), dt=1e-6, species=sp,
                              grid_type=abi.GRID_GENERALIZED, mode=abi.MODE_MIXED)
        U0 = initial_conditions(cfg, abi.IC_MIXING_3D, 3, p_ambient=1e5, T_ambient=300.0,
                                nkernels=3)
        X = wavy_nodes(cfg, amp=0.2)
    else:
        mode = abi.MODE_HYBRID if case == "hybrid3d" else abi.MODE_MIXED
        cfg = abi.make_config(3, (33, 20, 18), dt=5e-7, species=sp, visc=True, ceq=True,
                              mode=mode)
        U0 = initial_conditions(cfg, abi.IC_MIXING_3D, 3, p_ambient=1e5, T_ambient=300.0,
                                nkernels=3)

    def run(canary):
        monkeypatch.setenv("FST_DEBUG_CANARY", "1" if canary else "0")
        s = Solver(cfg)
        s.set_state(U0)
        if X is not None:
            s.apply_bcs()
            s.set_grid(X)
        s.rk_step(2)
        U = s.get_state()
        s.close()
        return U

    Un, Uc = run(False), run(True)
    assert np.isfinite(Uc).all() and np.array_equal(Un, Uc)


@pytest.mark.parametrize("mode", [abi.MODE_MIXED, abi.MODE_HYBRID])
def test_fused_stages_equal_unfused_bit_for_bit(mode, monkeypatch):
    """Fused 3D stages compute the next stage's primitives in the species
    kernel's epilogue (interior) and a ghost-shell pass (after the boundary
    fill) instead of one primitive pass over every cell; both evaluate the
    same equation of state on the same state, so runs agree bit for bit,
    through a bare RHS evaluation and a set_state in between."""
    cfg = abi.make_config(3, (33, 17, 19), dt=1e-7, species=SP5, visc=True, ceq=True,
                          buoyancy=True, g=9.81, rho_ref=1.0, periodic=(False, True, False),
                          bcs=("outflow", "reflective", "outflow", "outflow", "hydrostatic",
                               "reflective"), mode=mode)
    U0 = initial_conditions(cfg, abi.IC_MIXING_3D, 17, p_ambient=1e5, T_ambient=300.0,
                            nkernels=4)

    def run(unfused):
        monkeypatch.setenv("FST_MIXED_UNFUSED", "1" if unfused else "0")
        s = Solver(cfg)
        s.set_state(U0)
        s.rk_step(3)
        R = s.compute_rhs()
        s.rk_step(1)
        U1 = s.get_state()
        s.set_state(U1)
        s.rk_step(2)
        out = s.get_state(), R
        s.close()
        return out

    (Uf, Rf), (Uu, Ru) = run(False), run(True)
    assert np.isfinite(Uf).all()
    assert np.array_equal(Rf, Ru) and np.array_equal(Uf, Uu)


def bench_case(n, mode=abi.MODE_MIXED):
    """The benchmark workload (five-species viscous mixing, C-equation) at n^3
    with its time step (0.25 dx / max(|u| + c) of the initial state)."""
    import bench
    cfg = abi.make_config(3, (n, n, n), dt=1.0, species=bench.SPECIES, visc=True, ceq=True,
                          kap=10.0, eps=0.4, alpha=40.0, mode=mode)
    U0 = initial_conditions(cfg, abi.IC_MIXING_3D, bench.SEED, **bench.IC_KW)
    cfg.dt = bench.bench_dt(cfg, U0)
    return cfg, U0


def test_mixed_benchmark_case_128_at_its_time_step():
    """The benchmark's own case and time step at 128^3, 10 steps: every field
    under the bar."""
    cfg, U0 = bench_case(128)
    check_fields(cfg, *run_pair(cfg, U0, 10), U0)
