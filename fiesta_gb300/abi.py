"""ctypes mirror of include/fst.h (the libfst C ABI).

The structs here must match the C declarations field for field; the CPU
test ``tests/test_abi.py`` checks their sizes against the library.
"""
import ctypes as C

FST_ABI_VERSION = 1
FST_MAX_SPECIES = 16

FST_OK = 0
FST_ERR_INVALID = -1
FST_ERR_OOM = -2
FST_ERR_CUDA = -3
FST_ERR_TIMEOUT = -4
FST_ERR_NONFINITE = -5
FST_ERR_UNSUPPORTED = -6
FST_ERR_SIZE = -7

# src/bc.hpp:31 of the reference: enum class BCType {outflow, reflective,
# noslip, hydrostatic}
BC_OUTFLOW = 0
BC_REFLECTIVE = 1
BC_NOSLIP = 2
BC_HYDROSTATIC = 3
BC_NAMES = {"outflow": BC_OUTFLOW, "reflective": BC_REFLECTIVE,
            "noslip": BC_NOSLIP, "hydrostatic": BC_HYDROSTATIC}

MODE_PLAIN_FP64 = 0
MODE_MIXED = 1
MODE_HYBRID = 2

GRID_CARTESIAN = 0
GRID_GENERALIZED = 1

SCHEME_WENO5 = 1
SCHEME_CENTERED4 = 2
SCHEME_QUICK = 3
SCHEME_NAMES = {"weno5": SCHEME_WENO5, "centered4": SCHEME_CENTERED4, "quick": SCHEME_QUICK}

IC_SHOCK_TUBE_2D = 1
IC_EXPANSION_3D = 2
IC_MIXING_3D = 3
IC_RT_2D = 4
IC_RANDOM_SMOOTH = 5

_D16 = C.c_double * FST_MAX_SPECIES


class FstConfig(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int),
        ("ndim", C.c_int),
        ("nci", C.c_int), ("ncj", C.c_int), ("nck", C.c_int),
        ("ng", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("dt", C.c_double),
        ("ns", C.c_int),
        ("R", C.c_double),
        ("gamma", _D16), ("M", _D16), ("mu", _D16),
        ("visc", C.c_int),
        ("ceq", C.c_int),
        ("kap", C.c_double), ("eps", C.c_double), ("alpha", C.c_double),
        ("buoyancy", C.c_int),
        ("g_accel", C.c_double), ("rho_ref", C.c_double),
        ("xper", C.c_int), ("yper", C.c_int), ("zper", C.c_int),
        ("bc_xmin", C.c_int), ("bc_xmax", C.c_int),
        ("bc_ymin", C.c_int), ("bc_ymax", C.c_int),
        ("bc_zmin", C.c_int), ("bc_zmax", C.c_int),
        ("mode", C.c_int),
        ("audit_every", C.c_int),
        ("classify_every", C.c_int),
        ("grid_type", C.c_int),
        ("scheme", C.c_int),
        ("reserved", C.c_int * 5),
    ]


class FstStats(C.Structure):
    _fields_ = [
        ("max_wave_speed", C.c_double),
        ("max_chat", C.c_double),
        ("last_step_ms", C.c_double),
        ("flagged_face_fraction", C.c_double),
        ("steps", C.c_int64),
        ("kernel_launches", C.c_int64),
        ("nonfinite", C.c_int),
        ("reserved", C.c_int * 7),
    ]


class FstKernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_int64), ("total_ms", C.c_double)]


class FstIcParams(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("seed", C.c_uint64),
        ("p_ambient", C.c_double), ("T_ambient", C.c_double),
        ("p_high", C.c_double),
        ("radius", C.c_double),
        ("noise", C.c_double),
        ("rho_heavy", C.c_double), ("rho_light", C.c_double),
        ("nkernels", C.c_int),
        ("reserved", C.c_int * 7),
    ]


class FstNoiseParams(C.Structure):
    """fst_noise_params: fiesta.noise.{dh, eta, coff, nt, mode}."""
    _fields_ = [("dh", C.c_double), ("eta", C.c_double), ("coff", C.c_double),
                ("nt", C.c_int), ("mode", C.c_int), ("reserved", C.c_int * 6)]


def make_config(ndim=3, n=(8, 8, 8), L=(1.0, 1.0, 1.0), dt=1e-6, species=None,
                R=8.314462, visc=False, ceq=False, kap=10.0, eps=0.4, alpha=40.0,
                buoyancy=False, g=9.81, rho_ref=0.0, periodic=(False, False, False),
                bcs=("outflow",) * 6, mode=MODE_PLAIN_FP64, audit_every=0, dx=None,
                classify_every=1, grid_type=GRID_CARTESIAN, scheme=SCHEME_WENO5):
    """Build an FstConfig from deck-like arguments.

    ``species`` is a list of dicts {gamma, M, mu} as in ``fiesta.species``.
    ``bcs`` is (xmin, xmax, ymin, ymax, zmin, zmax) by name.  Cell sizes are
    ``L[d] / n[d]`` unless ``dx`` gives them explicitly, as ``fiesta.grid.dx``.
    """
    cfg = FstConfig()
    cfg.abi_version = FST_ABI_VERSION
    cfg.ndim = ndim
    cfg.nci, cfg.ncj = int(n[0]), int(n[1])
    cfg.nck = int(n[2]) if ndim == 3 else 1
    cfg.ng = 3
    if dx is None:
        dx = [L[0] / n[0], L[1] / n[1], (L[2] / n[2]) if ndim == 3 else L[0] / n[0]]
    cfg.dx, cfg.dy = float(dx[0]), float(dx[1])
    cfg.dz = float(dx[2]) if ndim == 3 else float(dx[0])
    cfg.dt = float(dt)
    species = species or [dict(gamma=1.4, M=0.02896, mu=1.8e-5)]
    cfg.ns = len(species)
    cfg.R = float(R)
    for s, sp in enumerate(species):
        cfg.gamma[s] = float(sp["gamma"])
        cfg.M[s] = float(sp["M"])
        cfg.mu[s] = float(sp.get("mu", 0.0))
    cfg.visc = int(bool(visc))
    cfg.ceq = int(bool(ceq))
    cfg.kap, cfg.eps, cfg.alpha = float(kap), float(eps), float(alpha)
    cfg.buoyancy = int(bool(buoyancy))
    cfg.g_accel, cfg.rho_ref = float(g), float(rho_ref)
    cfg.xper, cfg.yper, cfg.zper = (int(bool(p)) for p in periodic)
    b = [BC_NAMES[x] if isinstance(x, str) else int(x) for x in bcs]
    (cfg.bc_xmin, cfg.bc_xmax, cfg.bc_ymin, cfg.bc_ymax, cfg.bc_zmin, cfg.bc_zmax) = b
    cfg.mode = mode
    cfg.audit_every = audit_every
    cfg.classify_every = classify_every
    cfg.grid_type = grid_type
    cfg.scheme = SCHEME_NAMES[scheme] if isinstance(scheme, str) else int(scheme)
    return cfg


def grid_dims(cfg):
    """(ni, nj, nk, 3) of the node-coordinate array of a generalized grid."""
    nk = cfg.nck + 1 if cfg.ndim == 3 else 1
    return cfg.nci + 1, cfg.ncj + 1, nk, 3


def metrics_dims(cfg):
    """(ngi, ngj, ngk, d, d) of the metric tensor array."""
    ngi, ngj, ngk, _ = dims(cfg)
    return ngi, ngj, ngk, cfg.ndim, cfg.ndim


def dims(cfg):
    """(ngi, ngj, ngk, nvt) of the state array for ``cfg``."""
    ng = cfg.ng
    ngi, ngj = cfg.nci + 2 * ng, cfg.ncj + 2 * ng
    ngk = cfg.nck + 2 * ng if cfg.ndim == 3 else 1
    nv = (4 if cfg.ndim == 3 else 3) + cfg.ns
    nvt = nv + (5 if cfg.ceq else 0)
    return ngi, ngj, ngk, nvt


def nv_of(cfg):
    return (4 if cfg.ndim == 3 else 3) + cfg.ns


def config_to_dict(cfg):
    """Plain-dict form of a config (for JSON fixtures)."""
    out = {}
    for name, _ in FstConfig._fields_:
        val = getattr(cfg, name)
        if name in ("gamma", "M", "mu"):
            out[name] = [float(x) for x in val][: cfg.ns]
        elif name == "reserved":
            continue
        else:
            out[name] = val
    return out


def config_from_dict(d):
    cfg = FstConfig()
    for name, _ in FstConfig._fields_:
        if name == "reserved" or name not in d:
            continue
        if name in ("gamma", "M", "mu"):
            for s, x in enumerate(d[name]):
                getattr(cfg, name)[s] = x
        else:
            setattr(cfg, name, d[name])
    return cfg
