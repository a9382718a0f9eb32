"""The batched 2D ensemble against the same cases run one at a time, and
against the FP64 oracle; the autotuner's JSON persistence."""
import json
import os

import numpy as np
import pytest

from fiesta_gb300 import abi
from fiesta_gb300.batch import Batch, rt_ensemble
from fiesta_gb300.solver import Solver
from oracle.oracle import Oracle
from tests.golden_io import interior, rel_l2

pytestmark = pytest.mark.gpu


def small_ensemble():
    cfgs, states = rt_ensemble(ncases=6, nmin=24, nmax=90, seed=5)
    # vary the boundary types across cases
    cfgs[1].xper = 0
    cfgs[1].bc_xmin = abi.BC_REFLECTIVE
    cfgs[1].bc_xmax = abi.BC_NOSLIP
    cfgs[2].bc_ymax = abi.BC_REFLECTIVE
    return cfgs, states


def test_batch_matches_single_case_runs():
    cfgs, states = small_ensemble()
    b = Batch(cfgs)
    for c, U in enumerate(states):
        b.set_state(c, U)
    b.rk_step(5)
    for c, (cfg, U0) in enumerate(zip(cfgs, states)):
        s = Solver(cfg)
        s.set_state(U0)
        s.rk_step(5)
        Us, Ub = s.get_state(), b.get_state(c)
        for v in range(abi.nv_of(cfg)):
            a, r = interior(cfg, Ub[..., v]), interior(cfg, Us[..., v])
            assert rel_l2(a, r) <= 1e-6, (c, v, rel_l2(a, r))


def test_batch_vs_fp64_oracle():
    cfgs, states = small_ensemble()
    b = Batch(cfgs)
    for c, U in enumerate(states):
        b.set_state(c, U)
    b.rk_step(5)
    for c, (cfg, U0) in enumerate(zip(cfgs, states)):
        ref = abi.config_from_dict(abi.config_to_dict(cfg))
        ref.mode = abi.MODE_PLAIN_FP64
        o = Oracle(ref)
        o.set_state(U0)
        o.rk_step(5)
        Uo, Ub = o.get_state(), b.get_state(c)
        for v in range(abi.nv_of(cfg)):
            a, r, z = (interior(cfg, X[..., v]) for X in (Ub, Uo, U0))
            if np.abs(z).max() > 0:
                assert rel_l2(a, r) <= 1e-5, (c, v, rel_l2(a, r))
            if np.abs(r - z).max() > 0:
                assert rel_l2(a - z, r - z) <= 2e-3, (c, v, rel_l2(a - z, r - z))


def test_batch_tune_persists_choice(tmp_path):
    cfgs, states = small_ensemble()
    b = Batch(cfgs)
    for c, U in enumerate(states):
        b.set_state(c, U)
    path = str(tmp_path / "tune.json")
    h = b.tune(path)
    assert h in (4, 8, 16)
    d = json.load(open(path))
    assert len(d["entries"]) == 1 and d["entries"][0]["tile_height"] == h
    assert set(d["entries"][0]["ms_per_step"]) == {"4", "8", "16"}
    # the stored choice is reused without timing, and the state was restored
    b2 = Batch(cfgs)
    assert b2.tune(path) == h
    assert np.array_equal(b.get_state(0), states[0])
    assert b.info()["launches_per_step"] >= 8
