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
    w, h, k = b.tune(path)
    assert w in (16, 32, 64) and h in (4, 8, 16) and w * h <= 512 and k >= 1
    d = json.load(open(path))
    assert len(d["entries"]) == 1
    e = d["entries"][0]
    assert (e["tile_width"], e["tile_height"], e["blocks_per_sm"]) == (w, h, k)
    shapes = {tuple(int(x) for x in key.split("x")[:2]) for key in e["ms_per_step"]}
    assert shapes == {(16, 4), (16, 8), (16, 16), (32, 4), (32, 8), (32, 16), (64, 4), (64, 8)}
    assert e["candidates"] == len(e["ms_per_step"]) > len(shapes)
    assert e["best_ms"] == pytest.approx(min(e["ms_per_step"].values()), rel=1e-4)
    assert e["worst_ms"] == pytest.approx(max(e["ms_per_step"].values()), rel=1e-4)
    i = b.info()
    assert i["tune_candidates"] == e["candidates"] and i["tune_worst_ms"] >= i["tune_best_ms"] > 0
    # the stored choice is reused without timing, and the state was restored
    b2 = Batch(cfgs)
    assert b2.tune(path) == (w, h, k)
    assert b2.info()["tune_best_ms"] == pytest.approx(e["best_ms"])
    assert np.array_equal(b.get_state(0), states[0])
    assert b.info()["launches_per_step"] >= 8
    # another ensemble gets its own entry beside the first
    b3 = Batch(cfgs[:3])
    for c in range(3):
        b3.set_state(c, states[c])
    b3.tune(path)
    assert len(json.load(open(path))["entries"]) == 2


@pytest.mark.parametrize("shape", [(16, 4), (16, 16), (32, 4), (32, 16), (64, 4), (64, 8)])
def test_batch_every_tile_shape_matches_the_default(shape):
    """Every shape the autotuner may pick gives the bits of the 32 x 8 tile
    (same per-face and per-cell arithmetic, only the work split differs), at
    one and at the full persistent block count."""
    cfgs, states = small_ensemble()
    ref = Batch(cfgs)
    for c, U in enumerate(states):
        ref.set_state(c, U)
    ref.set_tile(32, 8)
    ref.rk_step(3)
    for k in (1, 0):
        b = Batch(cfgs)
        for c, U in enumerate(states):
            b.set_state(c, U)
        b.set_tile(*shape, k)
        i = b.info()
        assert (i["tile_width"], i["tile_height"]) == shape
        assert i["blocks_per_sm"] == (1 if k == 1 else i["max_blocks_per_sm"])
        b.rk_step(3)
        for c in range(len(cfgs)):
            assert np.array_equal(b.get_state(c), ref.get_state(c)), (shape, k, c)


def test_batch_rejects_shapes_it_has_no_kernel_for():
    cfgs, states = small_ensemble()
    b = Batch(cfgs)
    for bad in [(64, 16), (8, 8), (32, 2), (128, 4)]:
        with pytest.raises(Exception):
            b.set_tile(*bad)
    with pytest.raises(Exception):
        b.set_tile(32, 8, -1)
