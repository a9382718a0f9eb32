"""Restart files (fiesta_gb300/restart.py): the content of FIESTA's restart
(src/block.cpp:302-403, src/reader.cpp:33-120) as raw FP64 + JSON sidecar.
CPU tests use a stand-in for the solver's state accessors; the GPU test
restarts a run and checks that it continues bit for bit."""
import json

import numpy as np
import pytest

from fiesta_gb300 import abi, restart


class FakeSolver:
    def __init__(self, cfg, U=None):
        self.cfg = cfg
        self.U = U

    def get_state(self):
        return self.U.copy(order="F")

    def set_state(self, U):
        self.U = np.array(U, order="F")


def _cfg(ndim=3):
    sp = [dict(gamma=1.4, M=0.029, mu=1.8e-5), dict(gamma=1.67, M=0.004, mu=2e-5)]
    n = (7, 5, 4) if ndim == 3 else (9, 6)
    return abi.make_config(ndim, n, species=sp, ceq=True)


@pytest.mark.parametrize("ndim", [2, 3])
def test_round_trip_interior_bitwise(tmp_path, ndim):
    cfg = _cfg(ndim)
    rng = np.random.default_rng(5)
    U = np.asfortranarray(rng.standard_normal(abi.dims(cfg)))
    p = str(tmp_path / "restart-0000010.bin")
    restart.write_restart(p, FakeSolver(cfg, U), 10, 1.5e-3, title="box",
                          species_names=["Air", "He"])
    meta = json.load(open(p + ".json"))
    assert meta["restart_file_version"] == 2
    names = [d["name"] for d in meta["datasets"]]
    assert names[ndim + 1] == "/Solution/Air Density" and names[-1].startswith("/Solution/")
    s = FakeSolver(cfg, np.zeros(abi.dims(cfg), order="F"))
    t, time, title = restart.read_restart(p, s)
    assert (t, time, title) == (10, 1.5e-3, "box")
    ng = cfg.ng
    inner = (slice(ng, -ng), slice(ng, -ng)) + ((slice(ng, -ng),) if ndim == 3 else (slice(None),))
    assert np.array_equal(s.U[inner], U[inner])
    mask = np.ones(abi.dims(cfg)[:3], bool)
    mask[inner] = False
    assert np.all(s.U[mask] == 0.0)  # ghosts are not stored
    assert restart.read_restart(p, s, reset=True, time_index=3, time=0.5)[:2] == (3, 0.5)


def test_rejects_version_grid_and_missing(tmp_path):
    cfg = _cfg(3)
    U = np.zeros(abi.dims(cfg), order="F")
    p = str(tmp_path / "r.bin")
    restart.write_restart(p, FakeSolver(cfg, U), 0, 0.0)
    meta = json.load(open(p + ".json"))
    meta["restart_file_version"] = 1
    json.dump(meta, open(p + ".json", "w"))
    with pytest.raises(ValueError, match="version 1"):
        restart.read_restart(p, FakeSolver(cfg, U))
    meta["restart_file_version"] = 2
    json.dump(meta, open(p + ".json", "w"))
    other = abi.make_config(3, (8, 5, 4), species=[dict(gamma=1.4, M=0.029)] * 2, ceq=True)
    with pytest.raises(ValueError, match="grid"):
        restart.read_restart(p, FakeSolver(other, np.zeros(abi.dims(other), order="F")))
    with pytest.raises(FileNotFoundError):
        restart.read_restart(str(tmp_path / "none.bin"), FakeSolver(cfg, U))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [abi.MODE_PLAIN_FP64, abi.MODE_MIXED])
def test_restarted_run_continues_bitwise(tmp_path, mode):
    from fiesta_gb300.solver import Solver, initial_conditions
    sp = [dict(gamma=1.4, M=0.029, mu=1.8e-5), dict(gamma=1.67, M=0.004, mu=2e-5)]
    cfg = abi.make_config(3, (16, 12, 10), dt=1e-7, species=sp, visc=True, ceq=True, mode=mode)
    U0 = initial_conditions(cfg, abi.IC_MIXING_3D, 9, p_ambient=1e5, T_ambient=300.0,
                            nkernels=3)
    a = Solver(cfg)
    a.set_state(U0)
    a.rk_step(3)
    p = str(tmp_path / "restart.bin")
    restart.write_restart(p, a, 3, 3e-7)
    a.rk_step(2)
    b = Solver(cfg)
    assert restart.read_restart(p, b)[:2] == (3, 3e-7)
    b.rk_step(2)
    assert np.array_equal(a.get_state(), b.get_state())
