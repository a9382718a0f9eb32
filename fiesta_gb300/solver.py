"""Python binding of libfst (include/fst.h) and a host-side mirror of the
reference's module interface.

``Solver`` wraps one ``fst_ctx``.  ``Cart3D`` / ``Cart2D`` keep the method
names and call order of the reference's ``rk_func`` subclasses
(src/rkfunction.hpp:36-69, src/cart3d.cpp, src/cart2d.cpp) so that driver
code written against them reads the same:

    f = Cart3D(cfg, noise=np_) # cart3d_func(cf); np_: fiesta.noise or None
    f.var = U0                 # loadInitialConditions
    f.preSim()
    for t in range(tstart, tend + 1):   # src/main.cpp:61, inclusive
        f.preStep(); rkAdvance(cfg, f); f.postStep()   # postStep: noise filter

There is no CPU fallback: if libfst.so is missing or no GPU is present the
constructor raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .build import LIB, build, up_to_date

_lib = None

_EXPORTS = {
    # name: (restype, argtypes)
    "fst_config_defaults": (None, [C.POINTER(abi.FstConfig)]),
    "fst_state_size": (C.c_size_t, [C.POINTER(abi.FstConfig)]),
    "fst_nvt": (C.c_int, [C.POINTER(abi.FstConfig)]),
    "fst_create": (C.c_int, [C.POINTER(abi.FstConfig), C.POINTER(C.c_void_p)]),
    "fst_destroy": (None, [C.c_void_p]),
    "fst_last_error": (C.c_char_p, [C.c_void_p]),
    "fst_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fst_synchronize": (C.c_int, [C.c_void_p]),
    "fst_set_state": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_size_t]),
    "fst_get_state": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_size_t]),
    "fst_set_state_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "fst_get_state_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "fst_apply_bcs": (C.c_int, [C.c_void_p]),
    "fst_compute_rhs": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_size_t]),
    "fst_rk_step": (C.c_int, [C.c_void_p, C.c_int]),
    "fst_rk_step_get_state": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_size_t]),
    "fst_secondary": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_size_t]),
    "fst_check_finite": (C.c_int, [C.c_void_p]),
    "fst_fp64_rate": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "fst_noise_filter": (C.c_int, [C.c_void_p, C.POINTER(abi.FstNoiseParams)]),
    "fst_grid_size": (C.c_size_t, [C.POINTER(abi.FstConfig)]),
    "fst_metrics_size": (C.c_size_t, [C.POINTER(abi.FstConfig)]),
    "fst_set_grid": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_size_t]),
    "fst_get_metrics": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_size_t]),
    "fst_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                             C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "fst_get_stats": (C.c_int, [C.c_void_p, C.POINTER(abi.FstStats)]),
    "fst_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "fst_kernel_times": (C.c_int, [C.c_void_p, C.POINTER(abi.FstKernelTime), C.c_int,
                                   C.POINTER(C.c_int)]),
    "fst_fill_initial_conditions": (C.c_int, [C.POINTER(abi.FstConfig), C.POINTER(abi.FstIcParams),
                                              C.POINTER(C.c_double), C.c_size_t]),
}


def lib():
    """Load fiesta_gb300/libfst.so (building it first if sources are newer).

    FST_LIB names another build of the same library to load instead (for
    A/B timing of build variants); no build check is made for it.
    """
    global _lib
    if _lib is None:
        path = os.environ.get("FST_LIB")
        if not path:
            path = LIB
            if not up_to_date():
                build()
        if not os.path.exists(path):
            raise RuntimeError(f"libfst.so not found at {path}; run __graft_entry__.build()")
        L = C.CDLL(path)
        for name, (res, args) in _EXPORTS.items():
            if os.environ.get("FST_LIB") and not hasattr(L, name):
                continue  # an older build of the library: bind what it has
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def fp64_rate(stream=None):
    """FP64 FMA throughput of the current device in GFLOP/s (fst_fp64_rate)."""
    out = C.c_double()
    rc = lib().fst_fp64_rate(C.c_void_p(stream) if stream else None, C.byref(out))
    if rc != 0:
        raise FstError(rc, "fst_fp64_rate failed")
    return out.value


class FstError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libfst error {code}: {msg}")
        self.code = code


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def initial_conditions(cfg, kind, seed=0, **kw):
    """Seeded initial state (fst_fill_initial_conditions), LayoutLeft array."""
    ic = abi.FstIcParams()
    ic.kind = kind
    ic.seed = seed
    for k, v in kw.items():
        setattr(ic, k, v)
    shape = abi.dims(cfg)
    U = np.zeros(shape, dtype=np.float64, order="F")
    rc = lib().fst_fill_initial_conditions(C.byref(cfg), C.byref(ic), _dptr(U), U.size)
    if rc != 0:
        raise FstError(rc, "fst_fill_initial_conditions")
    return U


class Solver:
    """One libfst context on the current CUDA device."""

    def __init__(self, cfg):
        L = lib()
        self.cfg = cfg
        self.shape = abi.dims(cfg)
        self.n = int(np.prod(self.shape))
        self._ctx = C.c_void_p()
        rc = L.fst_create(C.byref(cfg), C.byref(self._ctx))
        if rc != 0:
            raise FstError(rc, "fst_create failed (see stderr)")

    def _check(self, rc, what):
        if rc != 0:
            msg = lib().fst_last_error(self._ctx)
            raise FstError(rc, f"{what}: {msg.decode() if msg else ''}")

    def close(self):
        if self._ctx:
            lib().fst_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state ---------------------------------------------------------
    def set_state(self, U):
        U = np.asfortranarray(U, dtype=np.float64)
        if U.shape != self.shape:
            raise ValueError(f"state shape {U.shape} != {self.shape}")
        self._check(lib().fst_set_state(self._ctx, _dptr(U), self.n), "set_state")

    def get_state(self):
        U = np.zeros(self.shape, dtype=np.float64, order="F")
        self._check(lib().fst_get_state(self._ctx, _dptr(U), self.n), "get_state")
        return U

    def set_state_device(self, ptr):
        self._check(lib().fst_set_state_device(self._ctx, C.c_void_p(ptr), self.n), "set_state_device")

    def get_state_device(self, ptr):
        self._check(lib().fst_get_state_device(self._ctx, C.c_void_p(ptr), self.n), "get_state_device")

    # -- generalized grids ----------------------------------------------
    def set_grid(self, nodes):
        """Node coordinates (ni, nj, nk, 3) of a generalized grid; computes
        the metric tensor on every cell (loadGrid + preSim of gen2d/gen3d)."""
        X = np.asfortranarray(nodes, dtype=np.float64)
        if X.shape != abi.grid_dims(self.cfg):
            raise ValueError(f"grid shape {X.shape} != {abi.grid_dims(self.cfg)}")
        self._check(lib().fst_set_grid(self._ctx, _dptr(X), X.size), "set_grid")

    def metrics(self):
        out = np.zeros(abi.metrics_dims(self.cfg), dtype=np.float64, order="F")
        self._check(lib().fst_get_metrics(self._ctx, _dptr(out), out.size), "get_metrics")
        return out

    # -- the path ------------------------------------------------------
    def apply_bcs(self):
        self._check(lib().fst_apply_bcs(self._ctx), "apply_bcs")

    def compute_rhs(self, out=True):
        if not out:
            self._check(lib().fst_compute_rhs(self._ctx, None, 0), "compute_rhs")
            return None
        R = np.zeros(self.shape, dtype=np.float64, order="F")
        self._check(lib().fst_compute_rhs(self._ctx, _dptr(R), self.n), "compute_rhs")
        return R

    def rk_step(self, nsteps=1):
        self._check(lib().fst_rk_step(self._ctx, int(nsteps)), "rk_step")

    def rk_step_get_state(self, nsteps=1, out=None):
        """`nsteps` steps and the resulting state copied to host memory (out,
        a Fortran-ordered float64 array of the state's shape, or a new one);
        into page-locked memory the copy overlaps the end of the last step."""
        if out is None:
            out = np.zeros(self.shape, dtype=np.float64, order="F")
        if out.shape != self.shape or out.dtype != np.float64 or not out.flags.f_contiguous:
            raise ValueError("out must be a Fortran-ordered float64 array of the state's shape")
        self._check(lib().fst_rk_step_get_state(self._ctx, int(nsteps), _dptr(out), self.n),
                    "rk_step_get_state")
        return out

    def secondary(self):
        nf = 6 if self.cfg.ndim == 3 else 5
        out = np.zeros(self.shape[:3] + (nf,), dtype=np.float64, order="F")
        self._check(lib().fst_secondary(self._ctx, _dptr(out), out.size), "secondary")
        return out

    def status(self, secondary=True):
        """Interior (min, max) per state variable and, with ``secondary``,
        per secondary variable (velocity, p, T, rho), reduced on the device:
        ``(vmin, vmax, xmin, xmax)`` arrays (the last two None without)."""
        nvt = self.shape[3]
        nx = self.cfg.ndim + 3
        vmin, vmax = np.zeros(nvt), np.zeros(nvt)
        xmin = np.zeros(nx) if secondary else None
        xmax = np.zeros(nx) if secondary else None
        nul = C.POINTER(C.c_double)()
        self._check(lib().fst_status(self._ctx, _dptr(vmin), _dptr(vmax),
                                     _dptr(xmin) if secondary else nul,
                                     _dptr(xmax) if secondary else nul), "status")
        return vmin, vmax, xmin, xmax

    def noise_filter(self, dh, eta, coff=0.0, nt=1, mode=1):
        """The postStep noise filter (fiesta.noise.*) on the current state."""
        np_ = abi.FstNoiseParams(dh=dh, eta=eta, coff=coff, nt=nt, mode=mode)
        self._check(lib().fst_noise_filter(self._ctx, C.byref(np_)), "noise_filter")

    def check_finite(self):
        rc = lib().fst_check_finite(self._ctx)
        if rc == abi.FST_ERR_NONFINITE:
            return False
        self._check(rc, "check_finite")
        return True

    def synchronize(self):
        self._check(lib().fst_synchronize(self._ctx), "synchronize")

    def set_stream(self, stream_ptr):
        self._check(lib().fst_set_stream(self._ctx, C.c_void_p(stream_ptr)), "set_stream")

    def set_profiling(self, on=True):
        self._check(lib().fst_set_profiling(self._ctx, int(bool(on))), "set_profiling")

    def kernel_times(self):
        """{kernel name: (launches, total ms)} since the last call."""
        buf = (abi.FstKernelTime * 64)()
        n = C.c_int(0)
        self._check(lib().fst_kernel_times(self._ctx, buf, 64, C.byref(n)), "kernel_times")
        return {buf[q].name.decode(): (buf[q].launches, buf[q].total_ms) for q in range(n.value)}

    def stats(self):
        s = abi.FstStats()
        self._check(lib().fst_get_stats(self._ctx, C.byref(s)), "get_stats")
        return {k: getattr(s, k) for k, _ in abi.FstStats._fields_ if k != "reserved"}


class _RkFunc:
    """Mirror of the reference's rk_func (src/rkfunction.hpp:36-69)."""

    ndim = None

    def __init__(self, cfg, noise=None):
        if cfg.ndim != self.ndim:
            raise ValueError(f"{type(self).__name__} needs ndim={self.ndim}")
        self.cf = cfg
        self.solver = Solver(cfg)
        self.t = 0
        self.noise = noise  # abi.FstNoiseParams of fiesta.noise, or None (off)

    # var / dvar / varx as in the reference (host copies)
    @property
    def var(self):
        return self.solver.get_state()

    @var.setter
    def var(self, U):
        self.solver.set_state(U)

    @property
    def varx(self):
        return self.solver.secondary()

    def compute(self):
        """R(U) into dvar; 3D applies BCs first (src/cart3d.cpp:221)."""
        self.dvar = self.solver.compute_rhs()
        return self.dvar

    def preSim(self):
        if self.ndim == 2:
            self.solver.apply_bcs()  # src/cart2d.cpp:136-145

    def preStep(self):
        pass  # folded into rkAdvance below (2D BCs run inside fst_rk_step)

    def postStep(self):
        """The noise filter when fiesta.noise is on (src/cart3d.cpp:319-374,
        src/cart2d.cpp:257-307, src/gen2d.cpp:150-179); the secondary
        variables of an output step are ``varx``, read when writing."""
        if self.noise is not None:
            n = self.noise
            self.solver.noise_filter(n.dh, n.eta, n.coff, n.nt, n.mode)
        self.t += 1

    def postSim(self):
        self.solver.synchronize()


class _CartFunc(_RkFunc):
    def __init__(self, cfg, noise=None):
        if cfg.grid_type != abi.GRID_CARTESIAN:
            raise ValueError(f"{type(self).__name__} needs a cartesian grid (use Gen3D/Gen2D)")
        super().__init__(cfg, noise)


class Cart3D(_CartFunc):
    ndim = 3


class Cart2D(_CartFunc):
    ndim = 2


class _GenFunc(_RkFunc):
    """Mirror of gen3d_func / gen2d_func (src/gen3d.hpp, src/gen2d.hpp): the
    node coordinates go into ``grid`` (ni, nj, nk, 3) as loadGrid fills the
    module's view, preSim computes the metric tensor, and no step applies
    boundary conditions."""

    def __init__(self, cfg, noise=None):
        if cfg.grid_type != abi.GRID_GENERALIZED:
            raise ValueError(f"{type(self).__name__} needs grid_type = GRID_GENERALIZED")
        super().__init__(cfg, noise if cfg.ndim == 2 else None)  # gen3d: no noise filter
        self.grid = None

    def preSim(self):
        if self.grid is None:
            raise ValueError("set the grid node coordinates before preSim")
        self.solver.set_grid(self.grid)

    @property
    def metrics(self):
        return self.solver.metrics()


class Gen3D(_GenFunc):
    ndim = 3


class Gen2D(_GenFunc):
    ndim = 2


def module_for(cfg):
    """The module class src/main.cpp:40-50 picks for a configuration."""
    if cfg.grid_type == abi.GRID_GENERALIZED:
        return Gen3D if cfg.ndim == 3 else Gen2D
    return Cart3D if cfg.ndim == 3 else Cart2D


def _is_bad(v):
    """isBad (src/status.cpp:102-107)."""
    import math
    return not ((math.isfinite(v) and (v != 0.0 and abs(v) >= 2.2250738585072014e-308 or v == 0.0))
                and -1.0e200 < v < 1.0e200)


def _is_concern(v):
    """isConcern (src/status.cpp:109-114)."""
    return v < -1.0e16 or v > 1.0e16


def status_report(f, var_names=None, varx_names=None):
    """The statusCheck table (src/status.cpp:116-253) for a Cart2D/Cart3D or
    Solver: one line per variable with its interior min and max and a flag,
    'bad' (non-normal or beyond 1e200), 'concern' (beyond 1e16) or ''."""
    s = f.solver if hasattr(f, "solver") else f
    vmin, vmax, xmin, xmax = s.status(secondary=True)
    nd = s.cfg.ndim
    var_names = var_names or [f"var{v}" for v in range(len(vmin))]
    varx_names = varx_names or (["X-Velocity", "Y-Velocity", "Z-Velocity"][:nd]
                                + ["Pressure", "Temperature", "Total Density"])

    def flag(a):
        return "bad" if _is_bad(a) else ("concern" if _is_concern(a) else "")

    rows = []
    for names, lo, hi in ((var_names, vmin, vmax), (varx_names, xmin, xmax)):
        for n, a, b in zip(names, lo, hi):
            rows.append((n, float(a), float(b), flag(a), flag(b)))
    return rows


def rkAdvance(cf, f):
    """rkAdvance(cf, f) (src/rk.cpp:28-70), with the module's preStep BCs."""
    f.solver.rk_step(1)
