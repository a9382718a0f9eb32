"""Host transfers of the state: the fused upload (a kernel reads page-locked
host memory and computes the interior primitives on the way) and the step
whose download overlaps its last stage (fst_rk_step_get_state) give the bits
of the plain copies around fst_rk_step."""
import numpy as np
import pytest

from fiesta_gb300 import abi
from fiesta_gb300.solver import Solver, initial_conditions

pytestmark = pytest.mark.gpu

SP5 = [dict(gamma=g, M=m / 1000.0, mu=mu) for g, m, mu in
       zip([1.4, 1.67, 1.3, 1.32, 1.4], [28.96, 4.0, 44.0, 16.0, 2.0],
           [1.8e-5, 1.99e-5, 1.47e-5, 1.1e-5, 0.88e-5])]


def pinned_like(U):
    """A Fortran-ordered float64 array in page-locked memory (torch's
    cudaHostAlloc'd buffer), holding U."""
    import torch
    t = torch.empty(U.size, dtype=torch.float64, pin_memory=True)
    a = t.numpy().reshape(U.shape, order="F")
    a[...] = U
    return t, a


def case(ns, visc, ceq, mode=abi.MODE_MIXED, n=(40, 36, 28)):
    cfg = abi.make_config(3, n, dt=2e-7, species=SP5[:ns], visc=visc, ceq=ceq, kap=10.0,
                          eps=0.4, alpha=40.0, mode=mode)
    U0 = initial_conditions(cfg, abi.IC_MIXING_3D, 7 + ns, p_ambient=1e5, T_ambient=300.0,
                            nkernels=6)
    return cfg, U0


@pytest.mark.parametrize("ns,visc,ceq", [(5, True, True), (3, False, True), (1, True, False),
                                         (2, False, False)])
def test_fused_upload_gives_the_bits_of_the_copy(ns, visc, ceq):
    cfg, U0 = case(ns, visc, ceq)
    keep, Up = pinned_like(U0)
    a, b = Solver(cfg), Solver(cfg)
    a.set_profiling(True)
    a.set_state(Up)      # page-locked: the fused upload
    b.set_state(U0)      # pageable: the copy, then the full primitive pass
    assert "mupload3d" in a.kernel_times()
    assert np.array_equal(a.get_state(), U0)
    a.rk_step(3)
    b.rk_step(3)
    assert np.array_equal(a.get_state(), b.get_state())
    a.close()
    b.close()


@pytest.mark.parametrize("mode", [abi.MODE_MIXED, abi.MODE_HYBRID])
def test_step_with_overlapped_download_gives_the_bits_of_step_then_copy(mode):
    cfg, U0 = case(5, True, True, mode=mode)
    a, b = Solver(cfg), Solver(cfg)
    if mode == abi.MODE_HYBRID:
        from fiesta_gb300 import hybrid as H
        from fiesta_gb300.train_classifier import load_params
        params, meta = load_params()
        for s in (a, b):
            H.set_params(s, params, meta["threshold"])
    keep, out = pinned_like(np.zeros_like(U0))
    for s in (a, b):
        s.set_state(U0)
    for nsteps in (1, 2):
        got = a.rk_step_get_state(nsteps, out)
        b.rk_step(nsteps)
        ref = b.get_state()
        assert got is out and np.array_equal(out, ref), nsteps
    # into pageable memory (the copy follows the step), and a round trip of
    # fused upload + overlapped download, as a host-driven loop does it
    assert np.array_equal(a.rk_step_get_state(1), (b.rk_step(1), b.get_state())[1])
    a.set_state(out)
    b.set_state(np.array(out, order="F"))
    a.rk_step_get_state(1, out)
    b.rk_step(1)
    assert np.array_equal(out, b.get_state())
    a.close()
    b.close()


def test_overlapped_download_elsewhere_follows_the_step():
    """2D and plain FP64 contexts take the step, then the copy."""
    for cfg in [abi.make_config(2, (64, 48), dt=1e-4, species=[dict(gamma=1.4, M=1.0, mu=0.0)],
                                R=1.0, ceq=True, mode=abi.MODE_MIXED,
                                bcs=("outflow", "outflow", "reflective", "reflective",
                                     "outflow", "outflow")),
                case(2, True, True, mode=abi.MODE_PLAIN_FP64, n=(24, 20, 16))[0]]:
        kind = abi.IC_SHOCK_TUBE_2D if cfg.ndim == 2 else abi.IC_MIXING_3D
        U0 = initial_conditions(cfg, kind, 3)
        a, b = Solver(cfg), Solver(cfg)
        a.set_state(U0)
        b.set_state(U0)
        keep, out = pinned_like(np.zeros_like(U0))
        a.rk_step_get_state(2, out)
        b.rk_step(2)
        assert np.array_equal(out, b.get_state())
        a.close()
        b.close()


def test_rk_step_get_state_rejects_bad_arguments():
    cfg, U0 = case(2, False, False, n=(16, 16, 16))
    s = Solver(cfg)
    with pytest.raises(Exception):
        s.rk_step_get_state(1, np.zeros((3, 3), order="F"))
    with pytest.raises(Exception):
        s.rk_step_get_state(-1)
    s.close()
