"""The C++ host interface (include/fst_module.hpp): rk_func and the four
module classes over the C ABI, as a C++ host program of the reference would
use them.  CPU: the header and test programs compile and link against
libfst.so.  GPU: the programs run — the reference's BC known answers
(tests/cpp/module_bc.cpp), and time steps of a cartesian 3D and a
generalized 2D case (tests/cpp/module_step.cpp) bit for bit with the oracle.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from fiesta_gb300 import abi
from fiesta_gb300.build import LIB, build
from oracle.oracle import Oracle
from tests.golden_io import same

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _compile(name, outdir):
    build()
    exe = os.path.join(outdir, name)
    libdir = os.path.dirname(LIB)
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "cpp", name + ".cpp"),
           "-L", libdir, "-lfst", "-Wl,-rpath," + libdir, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.parametrize("name", ["module_bc", "module_step", "module_deck"])
def test_cpp_module_programs_compile_and_link(name, tmp_path):
    assert os.path.exists(_compile(name, str(tmp_path)))


@pytest.mark.gpu
def test_gpu_cpp_module_bc_known_answers(tmp_path):
    r = subprocess.run([_compile("module_bc", str(tmp_path))], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "module_bc: ok" in r.stdout


def _load(prefix, case):
    raw = open(f"{prefix}_{case}.cfg", "rb").read()
    assert len(raw) == C.sizeof(abi.FstConfig)
    cfg = abi.FstConfig.from_buffer_copy(raw)
    shape = abi.dims(cfg)

    def arr(tag, shp):
        return np.fromfile(f"{prefix}_{case}.{tag}", dtype="<f8").reshape(shp, order="F")
    return cfg, arr, shape


@pytest.mark.gpu
def test_gpu_cpp_module_steps_match_oracle(tmp_path):
    prefix = str(tmp_path / "run")
    r = subprocess.run([_compile("module_step", str(tmp_path)), prefix], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    cfg, arr, shape = _load(prefix, "cart3d")
    o = Oracle(cfg)
    o.set_state(arr("U0", shape))
    o.rk_step(2)
    assert same(arr("U1", shape), o.get_state())
    cfg, arr, shape = _load(prefix, "gen2d")
    o = Oracle(cfg)
    o.set_state(arr("U0", shape))
    o.set_grid(arr("X", abi.grid_dims(cfg)))
    o.rk_step(3)
    assert same(arr("U1", shape), o.get_state())


def test_deck_export_round_trip(tmp_path):
    """The exported config, state and grid read back as written."""
    from fiesta_gb300 import deck
    from tests.test_deck import DECK_GEN2D
    p = tmp_path / "wavy.lua"
    p.write_text(DECK_GEN2D)
    summary = deck.export(str(p), str(tmp_path / "wavy"))
    cfg = abi.FstConfig.from_buffer_copy(open(tmp_path / "wavy.cfg", "rb").read())
    d = deck.load(str(p))
    assert bytes(cfg) == bytes(d.config())
    X = np.fromfile(tmp_path / "wavy.X", dtype="<f8").reshape(abi.grid_dims(cfg), order="F")
    assert np.array_equal(X, d.grid_nodes(cfg))
    assert summary["state_shape"] == list(abi.dims(cfg))


NOISE_KEYS = ("\nfiesta.noise.enabled = true\nfiesta.noise.dh = {dh}\nfiesta.noise.eta = 1e-3\n"
              "fiesta.noise.coff = 0.05\n")


def _deck_text(which, noise):
    from tests.test_deck import DECK_3D, DECK_GEN2D
    text = DECK_3D.replace('mode = "mixed"', 'mode = "plain"') if which == "cart3d" else DECK_GEN2D
    if noise:  # postStep's noise filter after every step
        text += NOISE_KEYS.format(dh=1e-5 if which == "cart3d" else 0.0)
    return text


def test_deck_export_writes_noise_params(tmp_path):
    """fiesta.noise on: <prefix>.noise holds the raw fst_noise_params that
    fst::load_noise reads; off: no such file."""
    from fiesta_gb300 import deck
    for noise in (False, True):
        p = tmp_path / f"deck{int(noise)}.lua"
        p.write_text(_deck_text("cart3d", noise))
        pre = str(tmp_path / f"run{int(noise)}")
        summary = deck.export(str(p), pre)
        assert summary["noise"] is noise and os.path.exists(pre + ".noise") is noise
    raw = open(pre + ".noise", "rb").read()
    assert raw == bytes(deck.load(str(p)).noise_params())


@pytest.mark.gpu
@pytest.mark.parametrize("which,noise", [("cart3d", False), ("gen2d", False), ("cart3d", True),
                                         ("gen2d", True)])
def test_gpu_cpp_runs_an_exported_deck(which, noise, tmp_path):
    """deck.lua -> python -m fiesta_gb300.deck -> C++ module interface
    (preStep, rkAdvance, postStep with the deck's noise filter) -> the same
    state as the oracle on the same inputs."""
    p = tmp_path / "deck.lua"
    p.write_text(_deck_text(which, noise))
    prefix = str(tmp_path / "run")
    r = subprocess.run(["python", "-m", "fiesta_gb300.deck", str(p), prefix], cwd=ROOT,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([_compile("module_deck", str(tmp_path)), prefix, "2"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    cfg = abi.FstConfig.from_buffer_copy(open(prefix + ".cfg", "rb").read())
    shape = abi.dims(cfg)
    U0 = np.fromfile(prefix + ".U0", dtype="<f8").reshape(shape, order="F")
    U1 = np.fromfile(prefix + ".U1", dtype="<f8").reshape(shape, order="F")
    o = Oracle(cfg)
    o.set_state(U0)
    if cfg.grid_type == abi.GRID_GENERALIZED:
        o.set_grid(np.fromfile(prefix + ".X", dtype="<f8").reshape(abi.grid_dims(cfg), order="F"))
    if noise:
        from fiesta_gb300 import deck
        np_ = deck.load(str(p)).noise_params()
        for _ in range(2):
            o.rk_step(1)
            o.noise_filter(np_.dh, np_.eta, np_.coff, np_.nt, np_.mode)
    else:
        o.rk_step(2)
    assert same(U1, o.get_state())
