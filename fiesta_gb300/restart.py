"""Restart files: the conserved state of a run and its time index.

FIESTA writes restarts as HDF5 (blockWriter::write, src/block.cpp:302-403):
group /Solution holds one dataset per conserved variable, named as in the
module's varNames (src/cart3d.cpp:98-110, src/cart2d.cpp:51-65), over the
interior cells with i fastest; group /Properties carries time_index, time,
title, metadata and restart_file_version (FIESTA_RESTART_VERSION = 2,
src/fiesta.hpp:31).  readRestart (src/reader.cpp:33-120) refuses another
version, fills the interior of var (ghosts stay zero) and takes time_index
and time unless restart.reset is set.

HDF5 is not available to this package, so the same content is written as a
raw little-endian FP64 file (the datasets back to back, in varNames order,
each over the interior with i fastest) plus a JSON sidecar holding the
/Properties attributes, the dataset names, offsets and extents.  Values
round-trip bit for bit through fst_get_state / fst_set_state.
"""
import json
import os

import numpy as np

from . import abi

RESTART_VERSION = 2
FORMAT = "fiesta-restart-raw"


def var_names(cfg, species_names=None):
    """varNames of cart3d / cart2d for this configuration."""
    ns = cfg.ns
    species_names = species_names or [f"Species{s}" for s in range(ns)]
    if cfg.ndim == 3:
        names = ["X-Momentum", "Y-Momentum", "Z-Momentum", "Energy"]
        cnames = ["C", "C_hat", "C_1", "C_2", "C_3"]
    else:
        names = ["X-Momentum", "Y-Momentum", "Energy"]
        cnames = ["C", "C_hat", "Tau_1", "Tau_2", "Debug"]
    names += [f"{n} Density" for n in species_names[:ns]]
    if cfg.ceq:
        names += cnames
    return names


def _interior(cfg, U):
    ng = cfg.ng
    if cfg.ndim == 3:
        return U[ng:-ng, ng:-ng, ng:-ng, :]
    return U[ng:-ng, ng:-ng, :, :]


def write_restart(path, solver, time_index, time, title="", metadata="none",
                  species_names=None):
    """Write the solver's current state to ``path`` (+ ``path + '.json'``)."""
    cfg = solver.cfg
    U = solver.get_state()
    inner = _interior(cfg, U)
    names = var_names(cfg, species_names)
    if len(names) != U.shape[3]:
        raise ValueError("variable names do not match the state")
    cells = [int(cfg.nci), int(cfg.ncj)] + ([int(cfg.nck)] if cfg.ndim == 3 else [])
    ncell = int(np.prod(cells))
    datasets = []
    with open(path, "wb") as f:
        for v, name in enumerate(names):
            a = np.ascontiguousarray(inner[..., v].reshape(-1, order="F"), dtype="<f8")
            datasets.append({"name": f"/Solution/{name}", "offset": v * ncell * 8,
                             "count": ncell})
            f.write(a.tobytes())
    meta = {
        "format": FORMAT,
        "restart_file_version": RESTART_VERSION,
        "properties": {"time_index": int(time_index), "time": float(time), "title": title,
                       "metadata": metadata},
        "ndim": int(cfg.ndim), "cells": cells, "dtype": "<f8", "order": "i fastest",
        "datasets": datasets,
    }
    with open(path + ".json", "w") as f:
        json.dump(meta, f, indent=1)


def read_restart(path, solver, reset=False, time_index=0, time=0.0):
    """Load a restart into ``solver`` (interior from the file, ghosts zero).

    Returns (time_index, time, title): the file's, or the given ones when
    ``reset`` is set (restart.reset).  Raises on a missing file, another
    format version, or a grid or variable set that does not match."""
    if not os.path.exists(path) or not os.path.exists(path + ".json"):
        raise FileNotFoundError(f"Restart file '{path}' does not exist.")
    with open(path + ".json") as f:
        meta = json.load(f)
    if meta.get("format") != FORMAT:
        raise ValueError(f"'{path}' is not a {FORMAT} file")
    ver = meta.get("restart_file_version")
    if ver != RESTART_VERSION:
        raise ValueError(f"Cannot read restart file '{path}' with version {ver}. "
                         f"Only version {RESTART_VERSION} files are readable")
    cfg = solver.cfg
    cells = [int(cfg.nci), int(cfg.ncj)] + ([int(cfg.nck)] if cfg.ndim == 3 else [])
    if meta["cells"] != cells or meta["ndim"] != cfg.ndim:
        raise ValueError(f"restart grid {meta['cells']} does not match {cells}")
    nvt = abi.dims(cfg)[3]
    if len(meta["datasets"]) != nvt:
        raise ValueError(f"restart has {len(meta['datasets'])} variables, the run {nvt}")
    U = np.zeros(abi.dims(cfg), dtype=np.float64, order="F")
    inner = _interior(cfg, U)
    raw = np.fromfile(path, dtype="<f8")
    shape = inner.shape[:3]
    for v, d in enumerate(meta["datasets"]):
        o = d["offset"] // 8
        inner[..., v] = raw[o:o + d["count"]].reshape(shape, order="F")
    solver.set_state(U)
    p = meta["properties"]
    if reset:
        return int(time_index), float(time), p.get("title", "")
    return int(p["time_index"]), float(p["time"]), p.get("title", "")
