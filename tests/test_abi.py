"""CPU tests of the C-ABI boundary: the library loads, exports every symbol
include/fst.h declares, its structs match the Python mirror, and the host-side
failure paths (invalid config, size limit) return status codes without any GPU
call.  No kernels run here."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from fiesta_gb300 import abi
from fiesta_gb300.solver import initial_conditions, lib
from tests.golden_io import load_all, same

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HEADER = os.path.join(ROOT, "include", "fst.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fst_[a-z_0-9]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    L = lib()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_struct_layouts_match_header():
    src = r'''
    #include <stdio.h>
    #include <stddef.h>
    #include "fst.h"
    int main(void) {
      printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(fst_config), sizeof(fst_stats),
             sizeof(fst_ic_params), sizeof(fst_kernel_time), offsetof(fst_config, mode),
             offsetof(fst_config, mu), offsetof(fst_stats, steps));
      return 0;
    }'''
    with tempfile.TemporaryDirectory() as d:
        cpath = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(cpath, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), cpath, "-o", exe], check=True)
        got = [int(x) for x in subprocess.run([exe], capture_output=True, text=True).stdout.split()]
    want = [C.sizeof(abi.FstConfig), C.sizeof(abi.FstStats), C.sizeof(abi.FstIcParams),
            C.sizeof(abi.FstKernelTime), abi.FstConfig.mode.offset, abi.FstConfig.mu.offset,
            abi.FstStats.steps.offset]
    assert got == want


def test_state_size_and_nvt():
    L = lib()
    cfg = abi.make_config(3, (10, 9, 8), ceq=True, species=[dict(gamma=1.4, M=1.0)] * 5)
    assert L.fst_nvt(C.byref(cfg)) == 14
    assert L.fst_state_size(C.byref(cfg)) == 16 * 15 * 14 * 14
    cfg2 = abi.make_config(2, (10, 9), ceq=True, species=[dict(gamma=1.4, M=1.0)] * 2)
    assert L.fst_nvt(C.byref(cfg2)) == 10
    assert L.fst_state_size(C.byref(cfg2)) == 16 * 15 * 10


def _create(cfg):
    ctx = C.c_void_p()
    return lib().fst_create(C.byref(cfg), C.byref(ctx)), ctx


@pytest.mark.parametrize("field,value", [
    ("ndim", 4), ("ng", 2), ("nci", 0), ("ns", 0), ("ns", 17), ("dx", 0.0), ("dy", -1.0),
    ("bc_ymin", 7), ("mode", 9), ("abi_version", 99),
])
def test_invalid_config_rejected_before_any_gpu_call(field, value):
    cfg = abi.make_config(3, (8, 8, 8))
    setattr(cfg, field, value)
    rc, ctx = _create(cfg)
    assert rc == abi.FST_ERR_INVALID
    assert not ctx.value


def test_bad_gamma_rejected():
    cfg = abi.make_config(3, (8, 8, 8), species=[dict(gamma=1.0, M=1.0)])
    assert _create(cfg)[0] == abi.FST_ERR_INVALID


def test_device_size_limit_returns_oom(monkeypatch):
    # host-side fault injection: an artificial device-memory limit
    monkeypatch.setenv("FST_MAX_DEVICE_BYTES", "1000000")
    cfg = abi.make_config(3, (64, 64, 64), ceq=True, visc=True)
    rc, ctx = _create(cfg)
    assert rc == abi.FST_ERR_OOM
    assert not ctx.value


def test_null_arguments():
    L = lib()
    assert L.fst_create(None, None) == abi.FST_ERR_INVALID
    assert L.fst_rk_step(None, 1) == abi.FST_ERR_INVALID
    assert L.fst_set_state(None, None, 0) == abi.FST_ERR_INVALID
    assert L.fst_last_error(None) == b"null context"


def test_initial_conditions_reproduce_golden_inputs():
    # the seeded, libm-free IC generator gives the same bits the golden
    # vectors were made from (on any host)
    for c in load_all():
        ic = dict(c.meta["ic"])
        kind, seed = ic.pop("kind"), ic.pop("seed")
        U = initial_conditions(c.cfg, kind, seed, **ic)
        assert same(U, c.U0), c.name
        assert np.array_equal(U.view(np.uint64), c.U0.view(np.uint64)), c.name


def test_initial_conditions_reject_bad_args():
    cfg = abi.make_config(3, (4, 4, 4))  # one species: expansion needs two
    with pytest.raises(Exception):
        initial_conditions(cfg, abi.IC_EXPANSION_3D, 1)
    with pytest.raises(Exception):
        initial_conditions(cfg, 99, 1)
