"""The learned hybrid: training kernels against the float64 oracle, BF16
tensor-core inference against FP32, and an ablation that shows what the
trained network gains over routing without it."""
import numpy as np
import pytest

from fiesta_gb300 import abi, hybrid as H
from fiesta_gb300.solver import Solver, initial_conditions
from oracle import mlp_oracle as M
from tests.golden_io import interior, rel_l2

pytestmark = pytest.mark.gpu


def _data(n, seed):
    import torch
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1, 1, (n, M.NI)).astype(np.float32)
    y = (X[:, 0] * X[:, 5] + 0.3 * X[:, 12] > 0.1).astype(np.uint8)
    return X, y, torch.as_tensor(X, device="cuda"), torch.as_tensor(y, device="cuda")


def test_gradient_matches_float64_oracle():
    X, y, Xd, yd = _data(5000, 1)
    p = M.init_params(4).astype(np.float32)
    loss, g = H.grad(Xd, yd, p, pos_weight=2.5)
    lo, go = M.loss_grad(p.astype(np.float64), X.astype(np.float64), y, pos_weight=2.5)
    assert abs(loss - lo) <= 1e-5 * abs(lo) + 1e-6
    assert np.linalg.norm(g - go) <= 1e-4 * np.linalg.norm(go)


def test_forward_fp32_and_tensor_core_paths():
    X, y, Xd, yd = _data(4000, 2)
    p = M.init_params(5).astype(np.float32)
    ref = M.prob(p.astype(np.float64), X.astype(np.float64))
    f32 = H.forward(Xd, p, tensor_cores=False)
    tc = H.forward(Xd, p, tensor_cores=True)
    assert np.abs(f32 - ref).max() <= 1e-5
    # BF16 weights and activations, FP32 accumulation
    assert np.abs(tc - ref).max() <= 2e-2
    assert np.mean((tc > 0.5) == (ref > 0.5)) >= 0.97


def test_training_reduces_loss_and_learns_labels():
    X, y, Xd, yd = _data(60000, 3)
    p, losses = H.train(Xd, yd, epochs=6, lr=3e-3, batch=4096, pos_weight=1.0, seed=2)
    assert losses[-1] < 0.5 * losses[0]
    acc = np.mean((M.prob(p.astype(np.float64), X.astype(np.float64)) > 0.5) == (y > 0))
    assert acc >= 0.95


def _run(cfg, U0, steps, params=None, threshold=0.5):
    s = Solver(cfg)
    s.set_state(U0)
    if params is not None:
        H.set_params(s, params, threshold)
    s.rk_step(steps)
    return s, s.get_state()


def test_hybrid_ablation_and_audit():
    # train on a handful of small seeded runs of the five-species gas
    X, Y = H.generate_training_data(n_runs=8, n=24, snapshots=3, steps_between=5, seed=77)
    assert 0.001 < float(Y.float().mean()) < 0.6
    params, losses = H.train(X, Y, epochs=4, lr=3e-3, batch=8192, pos_weight=3.0, seed=1)
    assert losses[-1] < losses[0]
    # held-out case: expanding high-pressure bubble
    cfg, U0 = H.training_run(0, n=32, seed=999, mode=abi.MODE_MIXED)
    _, Uw = _run(cfg, U0, 12)                               # full WENO everywhere
    hcfg = abi.config_from_dict(abi.config_to_dict(cfg))
    hcfg.mode = abi.MODE_HYBRID
    hcfg.audit_every = 4
    sh, Uh = _run(hcfg, U0, 12, params, 0.5)                # trained classifier
    sl, Ul = _run(hcfg, U0, 12, H.always_linear_params())   # no network: all linear
    c = H.counts(sh)
    assert c["faces"] > 0 and 0.0 < c["weno_faces"] / c["faces"] < 0.95
    assert c["audit_faces"] > 0 and c["audit_missed"] <= c["audit_nonsmooth"]
    st = sh.stats()
    assert 0.0 < st["flagged_face_fraction"] < 0.95
    assert np.isfinite(Uh).all()
    lin_ok = np.isfinite(Ul).all()
    for v in (3, 4):  # energy, first species
        eh = rel_l2(interior(cfg, Uh[..., v]) - interior(cfg, U0[..., v]),
                    interior(cfg, Uw[..., v]) - interior(cfg, U0[..., v]))
        if lin_ok:
            el = rel_l2(interior(cfg, Ul[..., v]) - interior(cfg, U0[..., v]),
                        interior(cfg, Uw[..., v]) - interior(cfg, U0[..., v]))
            assert eh < 0.5 * el, (v, eh, el)
        assert eh < 0.2, (v, eh)


@pytest.mark.parametrize("n,steps", [(None, 10), (256, 10)])
def test_shipped_classifier_holds_the_bar(n, steps):
    """The classifier shipped in fiesta_gb300/classifier_params.json, at the
    benchmark's operating point (classification every 4 steps, full-WENO
    audit every 20), on the five-species mixing case: every state field
    within the bar of tests/accuracy.py against the FP64 oracle, at 48x40x32
    with a small step and on the benchmark case itself (256^3, its time
    step).  The bar depends on resolution: at 128^3 the x-momentum error of
    the linear-upwind faces reaches 1.06e-5 after 10 steps.""" 
    from fiesta_gb300.train_classifier import load_params
    from tests.accuracy import check_fields, run_pair
    from tests.test_gpu_mixed import SP5, bench_case
    got = load_params()
    assert got is not None, "fiesta_gb300/classifier_params.json is missing"
    params, meta = got
    if n is None:
        cfg = abi.make_config(3, (48, 40, 32), dt=2e-7, species=SP5, visc=True, ceq=True,
                              kap=10.0, eps=0.4, alpha=40.0, mode=abi.MODE_HYBRID)
        U0 = initial_conditions(cfg, abi.IC_MIXING_3D, 20261206, p_ambient=1e5,
                                T_ambient=300.0, nkernels=8)
    else:
        cfg, U0 = bench_case(n, abi.MODE_HYBRID)
    cfg.audit_every, cfg.classify_every = 20, 4

    def setup(s):
        H.set_params(s, params, meta["threshold"])

    check_fields(cfg, *run_pair(cfg, U0, steps, setup=setup), U0)
