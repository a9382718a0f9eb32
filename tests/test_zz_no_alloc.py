"""The allocation-free 2D right-hand side, fst_rhs2d_noalloc.

Some host programs own all device memory themselves (a pool reserved at
start-up, a legacy host that forbids allocation once running, a loop that
cannot pay for cudaMalloc's device-wide synchronisation) and so cannot create
an fst_ctx, which allocates.  fst_rhs2d_noalloc serves them: the caller passes
device input and output, and the work arrays live in a fixed array inside the
library.  These tests call it through the C ABI and check it against the
context-based fst_compute_rhs, bit for bit (the plain path's bar), on two
calls in a row with different states, so the second call runs on scratch
left over from the first.

This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from fiesta_gb300 import abi
from fiesta_gb300.solver import Solver, initial_conditions, lib
from tests.golden_io import same

pytestmark = pytest.mark.gpu


def _entry():
    L = lib()
    fn = L.fst_rhs2d_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(abi.FstConfig), C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    return fn


def _config():
    sp = [dict(gamma=1.4, M=1.0, mu=2.928e-5), dict(gamma=1.6, M=2.0, mu=2.928e-5)]
    return abi.make_config(2, (40, 30), L=(1.0, 0.75), dt=1e-4, species=sp, R=1.0, visc=True,
                           ceq=True, buoyancy=True, g=0.5, rho_ref=1.2,
                           periodic=(True, False, False),
                           bcs=("outflow", "outflow", "hydrostatic", "reflective", "outflow",
                                "outflow"))


def _with_ghosts(cfg, seed):
    """A state with its ghosts filled, and its RHS from the context API."""
    s = Solver(cfg)
    s.set_state(initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, seed))
    s.apply_bcs()
    U = s.get_state()
    return U, s.compute_rhs()


def test_noalloc_matches_context_rhs_twice():
    import torch
    fn = _entry()
    cfg = _config()
    n = int(np.prod(abi.dims(cfg)))
    d_U = torch.empty(n, dtype=torch.float64, device="cuda")
    d_R = torch.empty(n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    for seed in (11, 12):
        U, R_ref = _with_ghosts(cfg, seed)
        d_U.copy_(torch.from_numpy(U.ravel(order="F")))
        d_R.fill_(float("nan"))  # every element must be written
        rc = fn(C.byref(cfg), C.c_void_p(d_U.data_ptr()), C.c_void_p(d_R.data_ptr()), n,
                C.c_void_p(stream.cuda_stream))
        assert rc == abi.FST_OK
        torch.cuda.synchronize()
        R = d_R.cpu().numpy().reshape(abi.dims(cfg), order="F")
        assert same(R, R_ref), seed


def test_noalloc_inside_a_stream_capture_replays_bit_for_bit():
    """After the first call on the device, a call (C-equation on: its
    reduction words are set by a kernel, not a host copy) sits inside a CUDA
    graph capture in thread-local mode, and two replays give the context
    API's RHS bit for bit."""
    import torch
    fn = _entry()
    cfg = _config()
    n = int(np.prod(abi.dims(cfg)))
    U, R_ref = _with_ghosts(cfg, 13)
    d_U = torch.from_numpy(U.ravel(order="F").copy()).cuda()
    d_R = torch.empty(n, dtype=torch.float64, device="cuda")
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):  # the first call on the device, outside any capture
        assert fn(C.byref(cfg), C.c_void_p(d_U.data_ptr()), C.c_void_p(d_R.data_ptr()), n,
                  C.c_void_p(side.cuda_stream)) == abi.FST_OK
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, capture_error_mode="thread_local"):
        rc = fn(C.byref(cfg), C.c_void_p(d_U.data_ptr()), C.c_void_p(d_R.data_ptr()), n,
                C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == abi.FST_OK
    for _ in range(2):
        d_R.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        R = d_R.cpu().numpy().reshape(abi.dims(cfg), order="F")
        assert same(R, R_ref)


def test_noalloc_rejects_other_configs_and_null_pointers():
    """Host-side checks only: every case returns before any launch."""
    import torch
    fn = _entry()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    for kw in (dict(mode=abi.MODE_MIXED), dict(mode=abi.MODE_HYBRID),
               dict(grid_type=abi.GRID_GENERALIZED, dx=(1.0, 1.0, 1.0))):
        cfg = abi.make_config(2, (12, 10), species=[dict(gamma=1.4, M=1.0)], R=1.0, **kw)
        n = int(np.prod(abi.dims(cfg)))
        assert fn(C.byref(cfg), p, p, n, None) == abi.FST_ERR_UNSUPPORTED, kw
    cfg = abi.make_config(2, (12, 10), species=[dict(gamma=1.4, M=1.0)], R=1.0)
    n = int(np.prod(abi.dims(cfg)))
    assert fn(C.byref(cfg), None, p, n, None) == abi.FST_ERR_INVALID
    assert fn(C.byref(cfg), p, None, n, None) == abi.FST_ERR_INVALID
    assert fn(None, p, p, n, None) == abi.FST_ERR_INVALID
    assert fn(C.byref(cfg), p, p, n + 1, None) == abi.FST_ERR_SIZE


def test_noalloc_largest_mixture_at_the_cell_limit():
    """The most demanding 2D config that the cell limit admits (16 species,
    viscous, C-equation) fits the fixed array and matches the context RHS."""
    import torch
    fn = _entry()
    sp = [dict(gamma=1.3 + 0.02 * s, M=1.0 + 0.1 * s, mu=2.928e-5) for s in range(16)]
    cfg = abi.make_config(2, (122, 122), dt=1e-4, species=sp, R=1.0, visc=True, ceq=True)
    n = int(np.prod(abi.dims(cfg)))
    assert n // (abi.nv_of(cfg) + 5) == 128 * 128  # exactly FST_NOALLOC_MAX_CELLS cells
    U, R_ref = _with_ghosts(cfg, 13)
    d_U = torch.from_numpy(U.ravel(order="F")).cuda()
    d_R = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    rc = fn(C.byref(cfg), C.c_void_p(d_U.data_ptr()), C.c_void_p(d_R.data_ptr()), n,
            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == abi.FST_OK
    torch.cuda.synchronize()
    assert same(d_R.cpu().numpy().reshape(abi.dims(cfg), order="F"), R_ref)


def test_noalloc_rejects_oversize_and_3d():
    import torch
    fn = _entry()
    big = abi.make_config(2, (200, 200), species=[dict(gamma=1.4, M=1.0)], R=1.0)
    n = int(np.prod(abi.dims(big)))
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    assert fn(C.byref(big), C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), n,
              None) == abi.FST_ERR_SIZE
    three = abi.make_config(3, (8, 8, 8))
    n3 = int(np.prod(abi.dims(three)))
    assert fn(C.byref(three), C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), n3,
              None) == abi.FST_ERR_UNSUPPORTED
