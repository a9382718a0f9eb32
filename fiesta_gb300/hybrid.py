"""Python side of the learned hybrid (FST_MODE_HYBRID): training-data
collection from solver states, GPU training through the library's own
kernels (fst_mlp_*), and parameter installation.

Device buffers for training data are torch CUDA tensors (plumbing only; all
arithmetic runs in libfst's kernels).
"""
import ctypes as C
import math

import numpy as np

from . import abi
from .solver import FstError, Solver, initial_conditions, lib

NI, NH = 20, 32
NP = NH * NI + NH + NH * NH + NH + NH + 1


class HybridCounts(C.Structure):
    _fields_ = [("faces", C.c_int64), ("weno_faces", C.c_int64), ("audit_faces", C.c_int64),
                ("audit_nonsmooth", C.c_int64), ("audit_missed", C.c_int64)]


_SIGS = {
    "fst_hybrid_features": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_float,
                                      C.POINTER(C.c_size_t)]),
    "fst_mlp_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_float,
                               C.c_void_p, C.POINTER(C.c_float), C.c_void_p]),
    "fst_mlp_train_epoch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.POINTER(C.c_int), C.c_float, C.c_float,
                                      C.c_int, C.POINTER(C.c_float), C.c_void_p]),
    "fst_mlp_forward": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_int,
                                  C.c_void_p]),
    "fst_hybrid_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_float]),
    "fst_hybrid_get_counts": (C.c_int, [C.c_void_p, C.POINTER(HybridCounts), C.c_int]),
}


def _L():
    L = lib()
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype, fn.argtypes = res, args
    return L


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def init_params(seed=0):
    """He-initialised FP32 parameters (packed as include/fst.h describes)."""
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, math.sqrt(2.0 / NI), (NH, NI))
    W2 = rng.normal(0, math.sqrt(2.0 / NH), (NH, NH))
    w3 = rng.normal(0, math.sqrt(1.0 / NH), NH)
    return np.concatenate([W1.ravel(), np.zeros(NH), W2.ravel(), np.zeros(NH), w3, [0.0]]
                          ).astype(np.float32)


def always_linear_params():
    """A network whose output is always 0: every face takes the linear flux."""
    p = np.zeros(NP, dtype=np.float32)
    p[-1] = -100.0
    return p


def collect_features(solver, label_ratio=20.0):
    """(X [n, 20] float32, Y [n] uint8) CUDA tensors for every face of the
    solver's current state."""
    import torch
    n = 3 * (solver.cfg.nci + 1) * (solver.cfg.ncj + 1) * (solver.cfg.nck + 1 if solver.cfg.ndim == 3 else 1)
    X = torch.empty((n, NI), dtype=torch.float32, device="cuda")
    Y = torch.empty((n,), dtype=torch.uint8, device="cuda")
    cnt = C.c_size_t(0)
    torch.cuda.synchronize()
    solver._check(_L().fst_hybrid_features(solver._ctx, _ptr(X), _ptr(Y), n, label_ratio,
                                           C.byref(cnt)), "hybrid_features")
    return X[: cnt.value], Y[: cnt.value]


def grad(X, Y, params, pos_weight=1.0):
    import torch
    p = torch.as_tensor(np.asarray(params, dtype=np.float32), device="cuda")
    g = torch.empty(NP, dtype=torch.float32, device="cuda")
    loss = C.c_float(0)
    rc = _L().fst_mlp_grad(_ptr(X), _ptr(Y), X.shape[0], _ptr(p), pos_weight, _ptr(g),
                           C.byref(loss), _stream())
    if rc:
        raise FstError(rc, "fst_mlp_grad")
    return loss.value, g.cpu().numpy()


def forward(X, params, tensor_cores=False):
    import torch
    p = torch.as_tensor(np.asarray(params, dtype=np.float32), device="cuda")
    out = torch.empty(X.shape[0], dtype=torch.float32, device="cuda")
    rc = _L().fst_mlp_forward(_ptr(X), X.shape[0], _ptr(p), _ptr(out), int(bool(tensor_cores)),
                              _stream())
    if rc:
        raise FstError(rc, "fst_mlp_forward")
    return out.cpu().numpy()


def train(X, Y, params=None, epochs=5, lr=3e-3, batch=8192, pos_weight=3.0, seed=0):
    """Minibatch Adam with the library's training kernels; the sample order
    is reshuffled every epoch.  Returns (params, per-epoch mean losses)."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    p = torch.as_tensor(init_params(seed) if params is None else np.asarray(params, np.float32),
                        device="cuda").clone()
    m = torch.zeros(NP, dtype=torch.float32, device="cuda")
    v = torch.zeros(NP, dtype=torch.float32, device="cuda")
    step = C.c_int(0)
    losses = []
    for _ in range(epochs):
        perm = torch.randperm(X.shape[0], device="cuda", generator=g)
        Xs, Ys = X[perm].contiguous(), Y[perm].contiguous()
        loss = C.c_float(0)
        rc = _L().fst_mlp_train_epoch(_ptr(Xs), _ptr(Ys), X.shape[0], _ptr(p), _ptr(m), _ptr(v),
                                      C.byref(step), lr, pos_weight, batch, C.byref(loss),
                                      _stream())
        if rc:
            raise FstError(rc, "fst_mlp_train_epoch")
        losses.append(loss.value)
    return p.cpu().numpy(), losses


def set_params(solver, params, threshold=0.5):
    a = np.ascontiguousarray(params, dtype=np.float32)
    solver._check(_L().fst_hybrid_set_params(solver._ctx, a.ctypes.data_as(C.POINTER(C.c_float)),
                                             float(threshold)), "hybrid_set_params")


def counts(solver, reset=False):
    c = HybridCounts()
    solver._check(_L().fst_hybrid_get_counts(solver._ctx, C.byref(c), int(bool(reset))), "counts")
    return {k: getattr(c, k) for k, _ in HybridCounts._fields_}


SPECIES5 = [dict(gamma=g, M=m / 1000.0, mu=mu) for g, m, mu in
            zip([1.4, 1.67, 1.3, 1.32, 1.4], [28.96, 4.0, 44.0, 16.0, 2.0],
                [1.8e-5, 1.99e-5, 1.47e-5, 1.1e-5, 0.88e-5])]


def wave_speed(cfg, U):
    ng = cfg.ng
    I = U[ng:-ng, ng:-ng, ng:-ng] if cfg.ndim == 3 else U[ng:-ng, ng:-ng]
    s0 = cfg.ndim + 1
    rho = sum(I[..., s0 + s] for s in range(cfg.ns))
    Cp = sum(I[..., s0 + s] / rho * (cfg.gamma[s] * cfg.R / cfg.M[s] / (cfg.gamma[s] - 1)) for s in range(cfg.ns))
    Cv = sum(I[..., s0 + s] / rho * (cfg.R / cfg.M[s] / (cfg.gamma[s] - 1)) for s in range(cfg.ns))
    m2 = sum(I[..., d] ** 2 for d in range(cfg.ndim))
    p = (Cp / Cv - 1) * (I[..., cfg.ndim] - 0.5 * m2 / rho)
    return float((np.sqrt(np.maximum(Cp / Cv * p / rho, 0)) + np.sqrt(m2) / rho).max())


def training_run(k, n=48, seed=0, mode=abi.MODE_MIXED):
    """Config and initial state of seeded training run k: bubbles, shock
    tubes, Gaussian pressure mixing and smooth random fields in turn, all
    with the five-species gas of the benchmark case."""
    rng = np.random.default_rng(seed + 7919 * k)
    cfg = abi.make_config(3, (n, n, n), dt=1.0, species=SPECIES5, visc=True, ceq=True, kap=10.0,
                          eps=0.4, alpha=40.0, mode=mode)
    kind = k % 4
    if kind == 0:
        U = initial_conditions(cfg, abi.IC_EXPANSION_3D, seed + k, p_ambient=1e5, T_ambient=300.0,
                               p_high=float(10 ** rng.uniform(5.5, 7.0)),
                               radius=float(rng.uniform(0.1, 0.3)), noise=0.01)
    elif kind == 1:
        U = initial_conditions(cfg, abi.IC_SHOCK_TUBE_2D, seed + k)  # planar in 3D
    elif kind == 2:
        U = initial_conditions(cfg, abi.IC_MIXING_3D, seed + k, p_ambient=1e5, T_ambient=300.0,
                               nkernels=int(rng.integers(2, 9)))
    else:
        U = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, seed + k)
    # the C-equation source and diffusion are stiff on the slow smooth flow:
    # it needs a smaller CFL number to stay stable (as in the reference)
    cfl = 0.05 if kind == 3 else 0.4
    cfg.dt = cfl * cfg.dx / max(wave_speed(cfg, U), 1e-12)
    return cfg, U


def generate_training_data(n_runs=50, n=48, snapshots=4, steps_between=8, seed=1000,
                           label_ratio=20.0):
    """Features and labels of every face of `snapshots` states of each run
    (the first snapshot is the initial state), concatenated on the GPU."""
    import torch
    Xs, Ys = [], []
    for k in range(n_runs):
        cfg, U = training_run(k, n, seed)
        s = Solver(cfg)
        s.set_state(U)
        for q in range(snapshots):
            if q:
                s.rk_step(steps_between)
            if not s.check_finite():
                break  # an unstable run contributes no further snapshots
            X, Y = collect_features(s, label_ratio)
            Xs.append(X.clone())
            Ys.append(Y.clone())
        s.close()
    return torch.cat(Xs), torch.cat(Ys)
