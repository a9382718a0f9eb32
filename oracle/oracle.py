"""Python loaders for the CPU checkers.

TEST INFRASTRUCTURE ONLY — imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs, never by the product package.

* ``Oracle``: oracle/liboracle.so, the plain C++ restatement of the
  reference's FP64 path (oracle/fst_oracle.cpp).  Built by ``build()``
  below on any host (gcc, -ffp-contract=off, OpenMP).
* ``Reference``: oracle/_ref/libfiesta_ref.so, the reference's own sources
  compiled against the Kokkos shim (oracle/ref_build.sh).  Only exists where
  the reference tree is present.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libfiesta_ref.so")


def build(force=False):
    """Compile oracle/fst_oracle.cpp into oracle/liboracle.so."""
    src = os.path.join(HERE, "fst_oracle.cpp")
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)):
        return ORACLE_SO
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC",
           "-shared", src, "-o", ORACLE_SO + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


ORACLE_FMA_SO = os.path.join(HERE, "liboracle_fma.so")


def build_fma(force=False):
    """The same restatement compiled with multiply-add contraction on
    (-ffp-contract=fast, FMA instructions): the rounding an FP64 build with
    fused multiply-adds gives, as the reference's CUDA build gets from nvcc
    by default.  Tests use the spread between the two FP64 builds as the
    floor of what any non-bitwise implementation can hold."""
    import platform
    src = os.path.join(HERE, "fst_oracle.cpp")
    if (not force and os.path.exists(ORACLE_FMA_SO)
            and os.path.getmtime(ORACLE_FMA_SO) >= os.path.getmtime(src)):
        return ORACLE_FMA_SO
    cxx = os.environ.get("CXX", "g++")
    arch = ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=fast", *arch, "-fopenmp", "-fPIC",
           "-shared", src, "-o", ORACLE_FMA_SO + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(ORACLE_FMA_SO + ".tmp", ORACLE_FMA_SO)
    return ORACLE_FMA_SO


def build_reference():
    """Compile the reference sources into oracle/_ref (no-op without them)."""
    subprocess.run(["bash", os.path.join(HERE, "ref_build.sh")], check=True)
    return REF_SO if os.path.exists(REF_SO) else None


def _dims(cfg):
    ng = cfg.ng
    ngi, ngj = cfg.nci + 2 * ng, cfg.ncj + 2 * ng
    ngk = cfg.nck + 2 * ng if cfg.ndim == 3 else 1
    nv = (4 if cfg.ndim == 3 else 3) + cfg.ns
    return ngi, ngj, ngk, nv + (5 if cfg.ceq else 0)


class _Checker:
    prefix = None
    _lib = None

    def __init__(self, cfg):
        lib = self._load()
        self.cfg = cfg
        self.shape = _dims(cfg)  # (ngi, ngj, ngk, nvt) LayoutLeft
        self.n = int(np.prod(self.shape))
        self.ctx = C.c_void_p()
        rc = getattr(lib, self.prefix + "create")(C.byref(cfg), C.byref(self.ctx))
        if rc != 0:
            raise RuntimeError(f"{self.prefix}create failed: {rc}")

    @classmethod
    def _load(cls):
        raise NotImplementedError

    def _call(self, name, *args):
        rc = getattr(self._lib, self.prefix + name)(self.ctx, *args)
        if rc != 0:
            raise RuntimeError(f"{self.prefix}{name} failed: {rc}")

    def __del__(self):
        try:
            if self.ctx:
                getattr(self._lib, self.prefix + "destroy")(self.ctx)
                self.ctx = C.c_void_p()
        except Exception:
            pass

    @staticmethod
    def _ptr(a):
        return a.ctypes.data_as(C.POINTER(C.c_double))

    def set_state(self, U):
        """U: float64 array of shape (ngi, ngj, ngk, nvt), Fortran order."""
        U = np.asfortranarray(U, dtype=np.float64)
        assert U.shape == self.shape
        self._call("set_state", self._ptr(U), C.c_size_t(self.n))

    def get_state(self):
        U = np.zeros(self.shape, dtype=np.float64, order="F")
        self._call("get_state", self._ptr(U), C.c_size_t(self.n))
        return U

    def apply_bcs(self):
        self._call("apply_bcs")

    def compute_rhs(self):
        R = np.zeros(self.shape, dtype=np.float64, order="F")
        self._call("compute_rhs", self._ptr(R), C.c_size_t(self.n))
        return R

    def rk_step(self, nsteps=1):
        self._call("rk_step", C.c_int(nsteps))

    def noise_filter(self, dh, eta, coff=0.0, nt=1, mode=1):
        """The postStep noise filter (serial loop order)."""
        from fiesta_gb300 import abi
        np_ = abi.FstNoiseParams(dh=dh, eta=eta, coff=coff, nt=nt, mode=mode)
        self._call("noise_filter", C.byref(np_))

    def noise(self):
        out = np.zeros(self.shape[:3], dtype=np.int32, order="F")
        self._call("get_noise", out.ctypes.data_as(C.POINTER(C.c_int)), C.c_size_t(out.size))
        return out

    def set_grid(self, nodes):
        """Node coordinates (ni, nj, nk, 3), Fortran order; computes the metrics."""
        X = np.asfortranarray(nodes, dtype=np.float64)
        self._call("set_grid", self._ptr(X), C.c_size_t(X.size))

    def metrics(self):
        d = self.cfg.ndim
        out = np.zeros(self.shape[:3] + (d, d), dtype=np.float64, order="F")
        self._call("get_metrics", self._ptr(out), C.c_size_t(out.size))
        return out

    def secondary(self):
        nf = 6 if self.cfg.ndim == 3 else 5
        shp = self.shape[:3] + (nf,)
        out = np.zeros(shp, dtype=np.float64, order="F")
        self._call("secondary", self._ptr(out), C.c_size_t(out.size))
        return out


class Oracle(_Checker):
    prefix = "orc_"

    @classmethod
    def _load(cls):
        if Oracle._lib is None:
            build()
            lib = C.CDLL(ORACLE_SO)
            lib.orc_set_threads.argtypes = [C.c_int]
            Oracle._lib = lib
        return Oracle._lib

    @classmethod
    def set_threads(cls, n):
        return cls._load().orc_set_threads(int(n))

    def last_max(self):
        a, b = C.c_double(), C.c_double()
        self._call("last_max", C.byref(a), C.byref(b))
        return a.value, b.value


class OracleFMA(_Checker):
    """The oracle built with fused multiply-adds (see build_fma)."""
    prefix = "orc_"

    @classmethod
    def _load(cls):
        if OracleFMA._lib is None:
            build_fma()
            lib = C.CDLL(ORACLE_FMA_SO)
            lib.orc_set_threads.argtypes = [C.c_int]
            lib.orc_set_threads(os.cpu_count() or 1)
            OracleFMA._lib = lib
        return OracleFMA._lib


class Reference(_Checker):
    prefix = "ref_"

    @staticmethod
    def available():
        return os.path.exists(REF_SO)

    @classmethod
    def _load(cls):
        if Reference._lib is None:
            if not os.path.exists(REF_SO):
                raise RuntimeError("reference checker not built (oracle/ref_build.sh)")
            Reference._lib = C.CDLL(REF_SO)
        return Reference._lib
