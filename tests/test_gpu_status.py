"""fst_status: device min/max of the state and the secondary variables over
the interior, against numpy over the host copies, with the reduction rules
of statusCheck (src/status.cpp:86-99, 155-235): strict comparisons against
+-DBL_MAX, so NaN is skipped and -inf (+inf) never becomes a maximum
(minimum)."""
import numpy as np
import pytest

from fiesta_gb300 import abi
from fiesta_gb300.solver import Solver, initial_conditions, status_report
from tests.golden_io import interior

pytestmark = pytest.mark.gpu

BIG = np.finfo(np.float64).max


def ref_minmax(a):
    a = np.asarray(a, dtype=np.float64).ravel()
    hi = a[a > -BIG]
    lo = a[a < BIG]
    return (lo.min() if lo.size else BIG), (hi.max() if hi.size else -BIG)


def check(s, cfg):
    U = s.get_state()
    X = s.secondary()
    vmin, vmax, xmin, xmax = s.status()
    for v in range(U.shape[3]):
        assert (vmin[v], vmax[v]) == ref_minmax(interior(cfg, U[..., v])), v
    for q in range(X.shape[3]):
        assert (xmin[q], xmax[q]) == ref_minmax(interior(cfg, X[..., q])), q


@pytest.mark.parametrize("mode", [abi.MODE_PLAIN_FP64, abi.MODE_MIXED])
def test_status_3d(mode):
    sp = [dict(gamma=1.4, M=0.029, mu=1.8e-5), dict(gamma=1.67, M=0.004, mu=2e-5)]
    cfg = abi.make_config(3, (20, 14, 11), dt=1e-7, species=sp, visc=True, ceq=True, mode=mode)
    s = Solver(cfg)
    s.set_state(initial_conditions(cfg, abi.IC_MIXING_3D, 3, p_ambient=1e5, T_ambient=300.0,
                                   nkernels=3))
    s.rk_step(2)
    check(s, cfg)
    rows = status_report(s)
    assert len(rows) == abi.dims(cfg)[3] + 6
    assert all(r[3] == "" and r[4] == "" for r in rows)


def test_status_2d_and_nonfinite():
    cfg = abi.make_config(2, (30, 18), dt=1e-4, species=[dict(gamma=1.4, M=1.0, mu=0.0)], R=1.0,
                          ceq=True)
    s = Solver(cfg)
    U = initial_conditions(cfg, abi.IC_SHOCK_TUBE_2D, 1)
    s.set_state(U)
    s.apply_bcs()
    check(s, cfg)
    # NaN skipped, +inf a maximum, -inf a minimum, never the other way
    U = s.get_state()
    U[5, 6, 0, 0] = np.nan
    U[7, 8, 0, 1] = np.inf
    U[9, 9, 0, 1] = -np.inf
    s.set_state(U)
    vmin, vmax, _, _ = s.status(secondary=False)
    assert (vmin[0], vmax[0]) == ref_minmax(interior(cfg, U[..., 0]))
    assert vmax[1] == np.inf and vmin[1] == -np.inf
    assert status_report(s)[1][3:] == ("bad", "bad")
