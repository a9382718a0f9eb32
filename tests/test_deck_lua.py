"""The deck read by the Lua 5.3 VM (include/fst_deck.h, libfst_deck.so) against
the Python reader (fiesta_gb300/deck.py) on the same decks: the run
configuration byte for byte, the noise parameters, the node coordinates of
generalized grids and the initial state from fiesta.initial_conditions bit
for bit, and the required-key errors.  A C++ program (tests/cpp/module_lua.cpp)
reads a deck through the C API with no Python and writes the configuration
and initial state; with a GPU it also steps the module (test_cpp_module-style
check against the oracle).  The library builds where Lua 5.3 sources are
present (a FIESTA tree's tpls/lua/src); elsewhere these tests skip."""
import ctypes as C
import glob
import os
import subprocess

import numpy as np
import pytest

from fiesta_gb300 import abi, deck

lua_deck = pytest.importorskip("fiesta_gb300.lua_deck")
if not lua_deck.available():
    pytest.skip("no Lua 5.3 sources to build libfst_deck.so", allow_module_level=True)

from tests.test_deck import DECK_3D, DECK_GEN2D, SAMPLES  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

DECK_NOISE_2D = """
fiesta.title = "rt"
fiesta.species = {{gamma=1.4, M=1.0, mu=1e-3}, {gamma=1.6, M=2.0, mu=1e-3}}
fiesta.eos.R = 1.0
fiesta.time.dt = 1e-4
fiesta.time.nt = 5
fiesta.grid.ndim = 2
fiesta.grid.ni = {12, 20}
fiesta.grid.dx = {1/12, 2/20}
fiesta.mpi.procs = {1, 1}
fiesta.bc.xperiodic = true
fiesta.bc.ymin = "hydrostatic"
fiesta.bc.ymax = "hydrostatic"
fiesta.viscosity.enabled = true
fiesta.buoyancy.enabled = true
fiesta.buoyancy.acceleration = 0.5
fiesta.buoyancy.rho_reference = 1.5
fiesta.ceq = {enabled = true, kappa = 2.0, epsilon = 0.4, alpha = 30, beta = 0, betae = 0}
fiesta.noise = {enabled = true, dh = 1e-3, eta = 0.1, coff = 0.5, nt = 2, mode = 1}
fiesta.gb300 = {mode = "MIXED", audit_every = 7, classify_every = 3}
function fiesta.initial_conditions(x, y, z, v)
    if v == 2 then return 2.5 + 0.1 * math.sin(6.283 * x) end
    if v == 3 then return y > 1 and 2.0 or 0.01 end
    if v == 4 then return y > 1 and 0.02 or 1.0 end
    return 0.01 * math.cos(3 * x + y)
end
"""


def _pair(tmp_path, text, name="deck.lua"):
    p = tmp_path / name
    p.write_text(text)
    return str(p), lua_deck.LuaDeck(str(p)), deck.load(str(p))


def _bytes(cfg):
    return bytes(C.string_at(C.addressof(cfg), C.sizeof(cfg)))


@pytest.mark.parametrize("text", [DECK_3D, DECK_GEN2D, DECK_NOISE_2D])
def test_lua_vm_reads_what_the_python_reader_reads(text, tmp_path):
    path, L, P = _pair(tmp_path, text)
    cfg = L.config()
    assert _bytes(cfg) == _bytes(P.config())
    npl, npp = L.noise_params(), P.noise_params()
    assert (npl is None) == (npp is None)
    if npl is not None:
        assert _bytes(npl) == _bytes(npp)
    X = None
    if cfg.grid_type == abi.GRID_GENERALIZED:
        X = L.grid_nodes(cfg)
        assert np.array_equal(X, P.grid_nodes(cfg))
    UL = L.initial_conditions(cfg, X)
    UP = P.initial_conditions(cfg, X)
    assert np.array_equal(UL.view(np.uint64), UP.view(np.uint64))


@pytest.mark.skipif(not os.path.isdir(SAMPLES), reason="reference sample decks not staged")
def test_reference_sample_decks_through_the_lua_vm():
    """The reference's own sample decks: the current-format ones give the
    Python reader's configuration; the legacy flat-global ones fail on their
    first required key in both."""
    ok = 0
    for p in sorted(glob.glob(os.path.join(SAMPLES, "*", "fiesta.lua"))):
        try:
            P = deck.load(p)
        except deck.DeckError as e:
            with pytest.raises(lua_deck.LuaDeckError):
                lua_deck.LuaDeck(p)
            continue
        L = lua_deck.LuaDeck(p)
        assert _bytes(L.config()) == _bytes(P.config()), p
        ok += 1
    assert ok >= 5


def test_required_key_errors(tmp_path):
    text = DECK_3D.replace("fiesta.time.dt = 1e-7\n", "")
    p = tmp_path / "nodt.lua"
    p.write_text(text)
    with pytest.raises(lua_deck.LuaDeckError, match="fiesta.time.dt"):
        lua_deck.LuaDeck(str(p))
    q = tmp_path / "syntax.lua"
    q.write_text("fiesta.title = \n")
    with pytest.raises(lua_deck.LuaDeckError, match="Cannot run config file"):
        lua_deck.LuaDeck(str(q))
    r = tmp_path / "badbc.lua"
    r.write_text(DECK_3D.replace('"reflective"', '"sticky"'))
    with pytest.raises(lua_deck.LuaDeckError, match="Unknown boundary condition 'sticky'"):
        lua_deck.LuaDeck(str(r))


def test_errors_inside_the_deck_functions_are_reported(tmp_path):
    """A deck function that fails, returns no number, or replaces the table
    `fiesta` gives an error status and message (no Lua panic)."""
    base = DECK_3D.split("function fiesta.initial_conditions")[0]
    cases = {
        "raises": ('function fiesta.initial_conditions(x, y, z, v) error("boom") end',
                   "error running function 'initial_conditions'"),
        "nonumber": ('function fiesta.initial_conditions(x, y, z, v) return "x" end',
                     "should return a number"),
        "replaced": ('function fiesta.initial_conditions(x, y, z, v) fiesta = 3; return 0 end',
                     "replaced the table 'fiesta'"),
    }
    for name, (fn, msg) in cases.items():
        p = tmp_path / f"{name}.lua"
        p.write_text(base + fn + "\n")
        d = lua_deck.LuaDeck(str(p))
        with pytest.raises(lua_deck.LuaDeckError, match=msg):
            d.initial_conditions(d.config())
        d.close()


def _compile_module_lua(outdir):
    from fiesta_gb300.build import DECK_LIB, LIB, build, build_deck, lua_sources
    build()
    build_deck()
    exe = os.path.join(outdir, "module_lua")
    libdir = os.path.dirname(LIB)
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "cpp", "module_lua.cpp"),
           "-L", libdir, "-lfst", "-l:" + os.path.basename(DECK_LIB),
           "-Wl,-rpath," + libdir, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.parametrize("text", [DECK_3D, DECK_GEN2D])
def test_cpp_program_reads_a_deck_with_no_python(text, tmp_path):
    exe = _compile_module_lua(str(tmp_path))
    p = tmp_path / "deck.lua"
    p.write_text(text)
    pre = str(tmp_path / "run")
    r = subprocess.run([exe, str(p), pre, "0"], capture_output=True, text=True)
    assert r.returncode == 0 and "module_lua: ok" in r.stdout, r.stdout + r.stderr
    raw = open(pre + ".cfg", "rb").read()
    cfg = abi.FstConfig.from_buffer_copy(raw)
    P = deck.load(str(p))
    assert raw == _bytes(P.config())
    U = np.fromfile(pre + ".U0", dtype="<f8").reshape(abi.dims(cfg), order="F")
    X = P.grid_nodes(cfg) if cfg.grid_type == abi.GRID_GENERALIZED else None
    assert np.array_equal(U, P.initial_conditions(cfg, X))


@pytest.mark.gpu
def test_gpu_cpp_program_steps_a_deck_like_the_oracle(tmp_path):
    """The deck runs end to end in C++ (Lua VM, module, steps) and equals the
    FP64 oracle bit for bit."""
    from oracle.oracle import Oracle
    from tests.golden_io import same
    exe = _compile_module_lua(str(tmp_path))
    p = tmp_path / "deck.lua"
    p.write_text(DECK_NOISE_2D.replace('mode = "MIXED"', 'mode = "plain"').replace(
        "fiesta.noise = {enabled = true", "fiesta.noise = {enabled = false"))
    pre = str(tmp_path / "run")
    r = subprocess.run([exe, str(p), pre, "3"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    cfg = abi.FstConfig.from_buffer_copy(open(pre + ".cfg", "rb").read())
    shape = abi.dims(cfg)
    U0 = np.fromfile(pre + ".U0", dtype="<f8").reshape(shape, order="F")
    U1 = np.fromfile(pre + ".U1", dtype="<f8").reshape(shape, order="F")
    o = Oracle(cfg)
    o.set_state(U0)
    o.apply_bcs()
    o.rk_step(3)
    assert same(U1, o.get_state())
