"""CPU: the float64 classifier oracle's gradient against finite differences
(pins the restatement the GPU training kernels are checked against)."""
import numpy as np

from oracle import mlp_oracle as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = M.init_params(1) + 0.05 * rng.standard_normal(M.NP)
    X = rng.uniform(-1, 1, (200, M.NI))
    y = (rng.uniform(size=200) < 0.3).astype(np.float64)
    _, g = M.loss_grad(p, X, y, pos_weight=3.0)
    idx = rng.choice(M.NP, 60, replace=False)
    h = 1e-6
    for q in idx:
        e = np.zeros(M.NP)
        e[q] = h
        lp, _ = M.loss_grad(p + e, X, y, 3.0)
        lm, _ = M.loss_grad(p - e, X, y, 3.0)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[q]) <= 1e-6 + 1e-4 * abs(fd), (q, fd, g[q])


def test_pack_roundtrip():
    p = M.init_params(2)
    assert np.array_equal(M.pack(*M.unpack(p)), p)
    assert M.NP == 20 * 32 + 32 + 32 * 32 + 32 + 32 + 1
