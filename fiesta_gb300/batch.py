"""Python binding of the batched 2D ensemble (fst_batch_* in include/fst.h)
and the seeded Rayleigh-Taylor / rising-bubble ensemble generator."""
import ctypes as C
import math

import numpy as np

from . import abi
from .solver import FstError, initial_conditions, lib


class BatchInfo(C.Structure):
    _fields_ = [("ncases", C.c_int), ("tile_height", C.c_int), ("tiles", C.c_int),
                ("persistent_blocks", C.c_int), ("launches_per_step", C.c_int),
                ("tile_width", C.c_int), ("interior_cells", C.c_int64),
                ("blocks_per_sm", C.c_int), ("max_blocks_per_sm", C.c_int),
                ("tune_candidates", C.c_int), ("reserved", C.c_int),
                ("tune_best_ms", C.c_double), ("tune_worst_ms", C.c_double)]


_SIGS = {
    "fst_batch_create": (C.c_int, [C.POINTER(abi.FstConfig), C.c_int, C.POINTER(C.c_void_p)]),
    "fst_batch_destroy": (None, [C.c_void_p]),
    "fst_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "fst_batch_set_state": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_size_t]),
    "fst_batch_get_state": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_size_t]),
    "fst_batch_rk_step": (C.c_int, [C.c_void_p, C.c_int]),
    "fst_batch_synchronize": (C.c_int, [C.c_void_p]),
    "fst_batch_stream": (C.c_void_p, [C.c_void_p]),
    "fst_batch_set_tile_height": (C.c_int, [C.c_void_p, C.c_int]),
    "fst_batch_set_tile": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "fst_batch_info": (C.c_int, [C.c_void_p, C.POINTER(BatchInfo)]),
    "fst_batch_tune": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int]),
}


def _L():
    L = lib()
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype, fn.argtypes = res, args
    return L


class Batch:
    """An ensemble of 2D mixed-precision cases stepped together."""

    def __init__(self, cfgs):
        L = _L()
        self.cfgs = list(cfgs)
        arr = (abi.FstConfig * len(self.cfgs))(*self.cfgs)
        self._b = C.c_void_p()
        rc = L.fst_batch_create(arr, len(self.cfgs), C.byref(self._b))
        if rc != 0:
            raise FstError(rc, "fst_batch_create failed (see stderr)")

    def _check(self, rc, what):
        if rc != 0:
            raise FstError(rc, f"{what}: {_L().fst_batch_last_error(self._b).decode()}")

    def close(self):
        if self._b:
            _L().fst_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, c, U):
        U = np.asfortranarray(U, dtype=np.float64)
        self._check(_L().fst_batch_set_state(self._b, c, U.ctypes.data_as(C.POINTER(C.c_double)),
                                             U.size), "set_state")

    def get_state(self, c):
        U = np.zeros(abi.dims(self.cfgs[c]), dtype=np.float64, order="F")
        self._check(_L().fst_batch_get_state(self._b, c, U.ctypes.data_as(C.POINTER(C.c_double)),
                                             U.size), "get_state")
        return U

    def rk_step(self, n=1):
        self._check(_L().fst_batch_rk_step(self._b, int(n)), "rk_step")

    def synchronize(self):
        self._check(_L().fst_batch_synchronize(self._b), "synchronize")

    @property
    def stream(self):
        return _L().fst_batch_stream(self._b)

    def set_tile_height(self, h):
        self._check(_L().fst_batch_set_tile_height(self._b, int(h)), "set_tile_height")

    def set_tile(self, width, height, blocks_per_sm=0):
        """RHS tile of width x height threads and persistent blocks per SM
        (0: the occupancy limit)."""
        self._check(_L().fst_batch_set_tile(self._b, int(width), int(height), int(blocks_per_sm)),
                    "set_tile")

    def tune(self, json_path=None, force=False):
        """Pick the fastest tile shape and blocks per SM on this ensemble;
        returns (width, height, blocks_per_sm)."""
        p = json_path.encode() if json_path else None
        self._check(_L().fst_batch_tune(self._b, p, int(bool(force))), "tune")
        i = self.info()
        return i["tile_width"], i["tile_height"], i["blocks_per_sm"]

    def info(self):
        i = BatchInfo()
        self._check(_L().fst_batch_info(self._b, C.byref(i)), "info")
        return {k: getattr(i, k) for k, _ in BatchInfo._fields_ if k != "reserved"}


def rt_ensemble(ncases=64, nmin=128, nmax=1024, seed=20261207, mode=abi.MODE_MIXED):
    """Configs and initial states of the batched Rayleigh-Taylor ensemble:
    square grids with n log-uniform in [nmin, nmax] on [0,1]^2, heavy/light
    density ratio uniform in [1.5, 3], gravity 9.81, two species, viscous,
    C-equation on, periodic in x, hydrostatic walls in y, interface perturbed
    by 8 seeded Fourier modes of total amplitude 1% of the width, dt from the
    acoustic CFL 0.5 of each case."""
    rng = np.random.default_rng(seed)
    cfgs, states = [], []
    for c in range(ncases):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        ratio = float(rng.uniform(1.5, 3.0))
        p0 = 1.0e5
        sp = [dict(gamma=1.4, M=1.0, mu=2.928e-5), dict(gamma=1.4, M=1.0 / ratio, mu=2.928e-5)]
        cmax = math.sqrt(1.4 * (p0 + ratio * 9.81) / 1.0)
        dt = 0.5 * (1.0 / n) / cmax
        cfg = abi.make_config(2, (n, n), L=(1.0, 1.0), dt=dt, species=sp, R=1.0, visc=True,
                              ceq=True, kap=10.0, eps=0.4, alpha=40.0, buoyancy=True, g=9.81,
                              rho_ref=0.0, periodic=(True, False, False),
                              bcs=("outflow", "outflow", "hydrostatic", "hydrostatic", "outflow",
                                   "outflow"), mode=mode)
        U = initial_conditions(cfg, abi.IC_RT_2D, seed + 1000 * c, rho_heavy=ratio,
                               rho_light=1.0, p_ambient=p0)
        cfgs.append(cfg)
        states.append(U)
    return cfgs, states
