"""The plain FP64 path against the oracle on the benchmark configurations
themselves, at their full sizes (bit for bit, which implies rel-L2 <= 1e-12):

  2D single-species shock tube, 400 x 400, WENO5 + C-equation, outflow in x,
  reflective in y, dt = 1e-4, 200 steps (the reference's own CPU-run case);
  3D two-species expansion, 256^3, viscous + C-equation, outflow, dt at
  CFL 0.5, two steps (the oracle takes seconds per step at this size; the
  properties that hold for any number of steps are checked in
  test_gpu_parity.test_gpu_full_size_periodic_conservation).
"""
import numpy as np
import pytest

from fiesta_gb300 import abi
from fiesta_gb300.solver import Solver, initial_conditions
from oracle.oracle import Oracle
from tests.golden_io import interior, rel_l2, same

pytestmark = pytest.mark.gpu


def _check(cfg, U0, steps):
    o, g = Oracle(cfg), Solver(cfg)
    o.set_state(U0)
    g.set_state(U0)
    o.rk_step(steps)
    g.rk_step(steps)
    Ug, Uo = g.get_state(), o.get_state()
    assert np.isfinite(Ug).all()
    assert same(Ug, Uo)
    for v in range(abi.nv_of(cfg)):
        assert rel_l2(interior(cfg, Ug[..., v]), interior(cfg, Uo[..., v])) <= 1e-12
    return Ug, U0


def test_shock_tube_400_200_steps():
    cfg = abi.make_config(2, (400, 400), dt=1e-4, species=[dict(gamma=1.4, M=1.0, mu=0.0)],
                          R=1.0, ceq=True, kap=10.0, eps=0.4, alpha=40.0,
                          bcs=("outflow", "outflow", "reflective", "reflective", "outflow",
                               "outflow"))
    U0 = initial_conditions(cfg, abi.IC_SHOCK_TUBE_2D, 1)
    Ug, _ = _check(cfg, U0, 200)
    # the shock has moved right of the diaphragm: density above the right state there
    ng = cfg.ng
    row = Ug[ng:-ng, 200 + ng, 0, 3]  # species-0 density along x, mid row
    assert row[:150].min() > 0.2 and row[-50:].max() < 0.2 and row[200:300].max() > 0.2


def test_expansion_256_two_steps():
    sp = [dict(gamma=1.4, M=0.02896, mu=1.8e-5), dict(gamma=1.67, M=0.004, mu=1.8e-5)]
    cfg = abi.make_config(3, (256, 256, 256), dt=1.0, species=sp, visc=True, ceq=True,
                          kap=10.0, eps=0.4, alpha=40.0)
    U0 = initial_conditions(cfg, abi.IC_EXPANSION_3D, 20261204, p_ambient=1e5,
                            T_ambient=300.0, p_high=1e7, radius=0.1, noise=0.01)
    # dt at CFL 0.5 from the initial max(|u| + c), as the configuration states
    ng = cfg.ng
    I = U0[ng:-ng, ng:-ng, ng:-ng]
    rho = I[..., 4] + I[..., 5]
    R = [cfg.R / cfg.M[s] for s in range(2)]
    cv = [R[s] / (cfg.gamma[s] - 1) for s in range(2)]
    gm1 = (I[..., 4] * R[0] + I[..., 5] * R[1]) / (I[..., 4] * cv[0] + I[..., 5] * cv[1])
    p = gm1 * I[..., 3]
    c = np.sqrt((1 + gm1) * p / rho)
    cfg.dt = 0.5 * cfg.dx / float(c.max())
    _check(cfg, U0, 2)


def test_expansion_256_twenty_steps():
    """The two-species expansion at 256^3 for 20 of its 100 steps, bit for
    bit (the oracle needs ~2.4 s per step at this size on the GPU host; every
    step of the plain path is the reference's arithmetic, so the remaining
    steps repeat what these check).  The reference has no adaptive time step:
    with dt at CFL 0.5 of the initial state (fluid at rest) the blast's
    wave speed doubles within two steps and the reference's own run diverges
    by step 6; dt = 0.5 dx / (2 S0) keeps CFL <= 0.5 against the largest
    wave speed the blast reaches (~2 S0)."""
    sp = [dict(gamma=1.4, M=0.02896, mu=1.8e-5), dict(gamma=1.67, M=0.004, mu=1.8e-5)]
    cfg = abi.make_config(3, (256, 256, 256), dt=1.0, species=sp, visc=True, ceq=True,
                          kap=10.0, eps=0.4, alpha=40.0)
    U0 = initial_conditions(cfg, abi.IC_EXPANSION_3D, 20261204, p_ambient=1e5,
                            T_ambient=300.0, p_high=1e7, radius=0.1, noise=0.01)
    import bench
    cfg.dt = 0.5 * cfg.dx / (2.0 * bench.max_wave_speed(cfg, U0))
    _check(cfg, U0, 20)


def test_mixing_384_mixed_step_vs_oracle():
    """The five-species mixing case at 384^3 (59 M cells, 390^3 x 14 state
    values): one mixed-precision step against the FP64 oracle, every field
    under the bar of tests/accuracy.py, finite, species masses conserved to
    the fluxes' accuracy."""
    from tests.accuracy import check_fields, run_pair
    from tests.test_gpu_mixed import bench_case
    cfg, U0 = bench_case(384)
    U, Ur, Up = run_pair(cfg, U0, 1)
    assert np.isfinite(U).all()
    check_fields(cfg, U, Ur, Up, U0)


def test_mixing_256_hundred_steps_mixed_vs_fp64():
    """The benchmark case itself (five-species mixing at 256^3, its time
    step) for 100 steps: the mixed path holds every field to the bar of
    tests/accuracy.py against the plain FP64 path over a full-length run,
    and stays finite."""
    from tests.accuracy import check_fields, run_pair
    from tests.test_gpu_mixed import bench_case
    cfg, U0 = bench_case(256)
    U, Ur, Up = run_pair(cfg, U0, 100, reference="plain")
    assert np.isfinite(U).all() and np.isfinite(Ur).all()
    for v, e, tol in check_fields(cfg, U, Ur, Up, U0):
        print(f"field {v}: rel-L2 {e:.3g} (bar {tol:.3g})")
