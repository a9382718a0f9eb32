"""Benchmark: Mcell-steps/s of the FIESTA RK2 step (RHS + update) on the
3D five-species viscous mixing case at 256^3 (C-equation on), one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--modes plain,mixed,hybrid] [--size 256]

A step is one time step of rkAdvance (src/rk.cpp:28-70): two RHS
evaluations, two stage combines and the ghost fills.  Inputs are synthetic
(the seeded compiled IC generator; the reference publishes no dataset), the
state (2 GB at 256^3) is far larger than L2, and dt is fixed from the initial
state as 0.5*dx/max(|u|+c).

Prints one JSON line.  `value` is the device-timed throughput with the state
resident in HBM; `e2e` is the same step driven through the C ABI with host
buffers (state uploaded from pinned memory and downloaded every step).
`--impl reference` times the reference's algorithm on the host cores instead
(the compiled reference sources where they were built, else the CPU oracle
restatement) and prints the same line with "impl": "reference".
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-steps/s 256^3 5-species viscous RK2 (FP64 plain / mixed / hybrid)"
def workload(n=256):
    return f"3D five-species viscous mixing, C-equation on, {n}^3 interior, outflow BCs"

SPECIES = [dict(gamma=g, M=m / 1000.0, mu=mu) for g, m, mu in
           zip([1.4, 1.67, 1.3, 1.32, 1.4], [28.96, 4.0, 44.0, 16.0, 2.0],
               [1.8e-5, 1.99e-5, 1.47e-5, 1.1e-5, 0.88e-5])]
SEED = 20261206
IC_KW = dict(p_ambient=1e5, T_ambient=300.0, nkernels=8)
MODES = {"plain": 0, "mixed": 1, "hybrid": 2}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def make_cfg(n, mode, dt=1.0):
    from fiesta_gb300 import abi
    return abi.make_config(3, (n, n, n), dt=dt, species=SPECIES, visc=True, ceq=True, kap=10.0,
                           eps=0.4, alpha=40.0, mode=mode)


# The time step of the workload: dt = DT_FACTOR dx / max(|u| + c) of the
# initial state, i.e. CFL 0.5 against twice the initial wave speed.  The
# blasts raise the largest wave speed to 1.4-1.8x its initial value within
# 50-200 steps; at 0.5 dx / S0 the FP64 path itself goes non-finite by step
# 80 at 128^3 (step 60 at 256^3), at 0.25 dx / S0 both paths stay finite over
# 200 steps at 128^3 and 256^3.
DT_FACTOR = 0.25


def bench_dt(cfg, U0):
    return DT_FACTOR * cfg.dx / max_wave_speed(cfg, U0)


def max_wave_speed(cfg, U):
    """max(|u| + c) over the interior, with the mixture gamma of the EOS."""
    ng = cfg.ng
    I = U[ng:-ng, ng:-ng, ng:-ng]
    rho = sum(I[..., 4 + s] for s in range(cfg.ns))
    Cp = sum(I[..., 4 + s] / rho * (cfg.gamma[s] * cfg.R / cfg.M[s] / (cfg.gamma[s] - 1))
             for s in range(cfg.ns))
    Cv = sum(I[..., 4 + s] / rho * (cfg.R / cfg.M[s] / (cfg.gamma[s] - 1)) for s in range(cfg.ns))
    gam = Cp / Cv
    ke = 0.5 * (I[..., 0] ** 2 + I[..., 1] ** 2 + I[..., 2] ** 2) / rho
    p = (gam - 1) * (I[..., 3] - ke)
    c = np.sqrt(gam * p / rho)
    u = np.sqrt(I[..., 0] ** 2 + I[..., 1] ** 2 + I[..., 2] ** 2) / rho
    return float((u + c).max())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled around the timed region.

    The sampler starts before the warm-up steps and polls every 50 ms; each
    sample is stamped on arrival, and the summary keeps the samples that fall
    inside the marked timed window (widened by one polling period on each
    side, so that a window shorter than the period still holds a sample).
    """

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 50

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []          # (arrival time, csv line)
        self.window = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 5.0:
                time.sleep(0.01)   # the first sample marks a running sampler
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def mark(self, t_start, t_end):
        self.window = (t_start, t_end)

    def __exit__(self, *a):
        if self.proc:
            time.sleep(2 * self.PERIOD_MS / 1e3)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        pad = self.PERIOD_MS / 1e3
        for t, ln in self.lines:
            if self.window and not (self.window[0] - pad <= t <= self.window[1] + pad):
                continue
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, flag in zip(names, parts[4:8]):
                if flag.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "period_ms": self.PERIOD_MS}


# Algorithmic bytes per launch of each kernel: the fields it must read and
# write once, counted over the cells it covers (FP64 = 8 B, FP32 = 4 B).
def algorithmic_bytes(kernel, cfg):
    nci, ncj, nck, ns = cfg.nci, cfg.ncj, cfg.nck, cfg.ns
    nv = 4 + ns
    nvt = nv + (5 if cfg.ceq else 0)
    ngi, ngj, ngk = nci + 6, ncj + 6, nck + 6
    allc = ngi * ngj * ngk
    faces = (nci + 1) * (ncj + 1) * (nck + 1)
    inner = nci * ncj * nck
    visc, ceq, buoy = bool(cfg.visc), bool(cfg.ceq), bool(cfg.buoyancy)
    tab = {
        # plain FP64 kernels (8-byte words)
        "prim3d": 8 * allc * (nv + 1 + 5 + ns + 1),
        "flux3d": 8 * faces * (nv + 4 + 3 * nv),
        "faces3d": 8 * faces * (3 + ns + 1 + 4 + 18 + 27),
        "cell3d": 8 * inner * (3 * nv + 6 + 18 + 27 + 5 + 2 * nvt),
        # mixed, the full primitive pass (all cells): FP64 state in; FP32 Q,
        # rho, velocity, the pressure pair, [mu], [e, C, the five pair low
        # parts] out, [FP64 rho]
        "mprim3d": allc * (8 * nvt + 4 * (nv + 1 + 3 + 2 + visc + (11 if ceq else 0))
                           + 8 * buoy),
        # cell terms of the momenta and energy: the pressure pair, u, v,
        # [FP64 rho]; old and new momenta and energy
        "mcell3d": inner * (8 + 8 + 8 * buoy + 16 * 4),
        # C-equation: u, v, w, rho, e, the five pair low parts, C0..4; old and
        # new C variables; the next stage's FP32 C variables (fused stages)
        "mceq3d": inner * (4 * (3 + 2 + 5 + 5) + 16 * 5 + 4 * 5) if ceq else 0,
        # species: Q_s, u, v, w; old and new state of the species
        "mspec3d": inner * (4 * (ns + 3) + 16 * ns),
        # momenta + energy faces: Q0..3, u, v, w, [mu], [rho, C1..4]; the
        # momenta and energy of U_new read and written
        "mmom3d": inner * (4 * (4 + 3 + visc + (5 if ceq else 0)) + 16 * 4),
    }
    # fused stages: the species kernel also reads the momenta and energy of
    # U_new and writes the next stage's primitives of the interior; the
    # ghost-shell pass covers the remaining cells
    prim_out = 4 * (nv + 1 + 3 + 2 + visc + (6 if ceq else 0)) + 8 * buoy
    tab["mspec3d_eos"] = tab["mspec3d"] + inner * (8 * 4 + prim_out)
    tab["mprim3d_shell"] = (allc - inner) * (8 * nvt + 4 * (nv + 1 + 3 + 2 + visc
                                                            + (11 if ceq else 0)) + 8 * buoy)
    # generalized grids (plain FP64): primitives read the 9 metrics and write
    # rho, p and the contravariant velocity; the cell pass reads the fluxes,
    # p and the 9 metrics once each
    if getattr(cfg, "grid_type", 0) == 1:
        tab["prim3d"] = 8 * allc * (nv + 9 + 5)
        tab["cell3d"] = 8 * inner * (3 * nv + 1 + 9 + 2 * nvt)
        # mixed: the pressure pair and 18 FP32 metric fields in, the momenta,
        # energy and C-variables old and new
        tab["gen_cell"] = inner * (4 * (2 + 18) + 16 * (4 + (nvt - nv)))
        tab["gen_tvel"] = allc * 4 * (3 + 9 + 3)
    tab["mspec3d_hybrid"] = tab["mspec3d"] + inner * 3
    tab["mspec3d_hybrid_eos"] = tab["mspec3d_eos"] + inner * 3
    tab["mmom3d_hybrid"] = tab["mmom3d"] + inner * 3
    return tab.get(kernel)


# DRAM read + write bytes per launch of the 3D mixed kernels on the 256^3
# benchmark case: an ncu capture (dram__bytes_read.sum + dram__bytes_write.sum)
# of each kernel on the same case at 128^3, scaled by the cells (x8).  ncu does
# not run inside the bench, so these are the captured figures, labelled so in
# the line.
TRAFFIC_BYTES_PER_LAUNCH_256 = {
    "mspec3d_eos": 4.078e9,
    "mmom3d": 1.936e9,
    "mceq3d": 2.807e9,
    "mcell3d": 1.167e9,
}


def read_traffic(kernel):
    """DRAM bytes per launch from the captured figures, if the kernel has one."""
    return TRAFFIC_BYTES_PER_LAUNCH_256.get(kernel)


def run_gpu_mode(mode_name, n, steps, warmup, U0, dt, peak_gbs, peak_kind, e2e_steps):
    import torch
    from fiesta_gb300 import abi
    from fiesta_gb300.solver import Solver, lib
    cfg = make_cfg(n, MODES[mode_name], dt)
    if mode_name == "hybrid":
        cfg.audit_every = 20    # a full-WENO audit step every 20 steps
        cfg.classify_every = 4  # the smoothness map is refreshed every 4 steps
    s = Solver(cfg)
    hyb = None
    if mode_name == "hybrid":
        from fiesta_gb300 import hybrid as H
        from fiesta_gb300.train_classifier import load_params
        got = load_params()
        if got is None:
            raise RuntimeError("fiesta_gb300/classifier_params.json missing: run "
                               "python -m fiesta_gb300.train_classifier")
        params, meta = got
        H.set_params(s, params, meta["threshold"])
        hyb = meta
    stream = torch.cuda.current_stream()
    s.set_stream(stream.cuda_stream)
    s.set_state(U0)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler() as clk:
        for _ in range(warmup):
            s.rk_step(1)
        torch.cuda.synchronize()
        l0 = s.stats()["kernel_launches"]
        s.set_profiling(True)
        s.kernel_times()
        torch.cuda.synchronize()
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            dist.barrier()  # ranks start the timed region together
        t_start = time.perf_counter()
        ev0.record(stream)
        for _ in range(steps):
            s.rk_step(1)
        ev1.record(stream)
        torch.cuda.synchronize()
        clk.mark(t_start, time.perf_counter())
    ms = ev0.elapsed_time(ev1)
    kt = s.kernel_times()
    s.set_profiling(False)
    launches = s.stats()["kernel_launches"] - l0
    cells = cfg.nci * cfg.ncj * cfg.nck
    value = cells * steps / (ms / 1e3) / 1e6
    finite = s.check_finite()
    U_final = s.get_state()  # after warmup + steps, for the accuracy report
    hybrid_info = None
    if hyb is not None:
        from fiesta_gb300 import hybrid as H
        c = H.counts(s)
        hybrid_info = {"weno_face_fraction": c["weno_faces"] / max(1, c["faces"]),
                       "audit_faces": c["audit_faces"],
                       "audit_nonsmooth": c["audit_nonsmooth"],
                       "audit_missed": c["audit_missed"],
                       "classifier": {k: hyb[k] for k in ("threshold", "label_ratio",
                                                           "train_faces", "val_weno_fraction",
                                                           "val_miss_rate")}}

    # dominant kernel and its live roofline
    top = max(kt.items(), key=lambda kv: kv[1][1]) if kt else None
    roof = None
    if top:
        name, (nl, tot) = top
        per_ms = tot / nl
        b = algorithmic_bytes(name, cfg)
        ach = b / (per_ms / 1e3) / 1e9 if b else None
        tr = read_traffic(name)
        roof = {"bound": "hbm", "kernel": name, "achieved": ach, "peak": peak_gbs, "unit": "GB/s",
                "frac": ach / peak_gbs if ach else None, "traffic": tr,
                "traffic_source": ("DRAM read + write bytes of a committed ncu capture of this "
                                   "kernel on the same case at 128^3, scaled by the cells "
                                   "(x8); not measured in this run") if tr else None,
                "algorithmic_bytes_per_launch": b, "avg_launch_ms": per_ms,
                "peak_source": peak_kind,
                "share_of_step": tot / ms}
        if mode_name == "plain":  # the FP64 pipe, not HBM, is this kernel's roof
            from fiesta_gb300.solver import fp64_rate
            roof["fp64_peak_gflops_measured"] = fp64_rate(stream.cuda_stream)
            roof["bound"] = "fp64"
            roof["bound_note"] = ("FP64 pipe 85 % busy, DRAM a few % (an ncu capture of "
                                  "k_flux3d at 64^3); the GB/s figures show how far below the "
                                  "HBM roof an FP64-bound kernel sits")

    # end to end through the C ABI with host buffers: upload, step, download.
    # fst_set_state from page-locked memory is the fused upload (3D mixed:
    # the primitives are computed as the state arrives) and
    # fst_rk_step_get_state copies each variable group out as soon as the
    # last stage has finished it.  One untimed round trip first; every timed
    # round trip is bracketed by events around the upload and around the
    # step + download.  The plain link rates (one copy each way) and a
    # round trip with plain copies around fst_rk_step are recorded beside it.
    n_state = int(np.prod(abi.dims(cfg)))
    host = torch.empty(n_state, dtype=torch.float64, pin_memory=True)
    host.numpy()[:] = np.asfortranarray(U0).ravel(order="F")
    L = lib()
    L.fst_rk_step_get_state.restype = C.c_int
    L.fst_rk_step_get_state.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_size_t]
    ptr = C.cast(C.c_void_p(host.data_ptr()), C.POINTER(C.c_double))

    def round_trip(ev=None):
        if ev:
            ev[0].record(stream)
        assert L.fst_set_state(s._ctx, ptr, n_state) == 0
        if ev:
            ev[1].record(stream)
        assert L.fst_rk_step_get_state(s._ctx, 1, ptr, n_state) == 0
        if ev:
            ev[2].record(stream)

    round_trip()
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(e2e_steps)]
    # the host calls are synchronous, so a pause of the Python host shows up
    # as device idle time: no garbage collection inside the timed loop (a C
    # or C++ caller of the same entry points has none)
    import gc
    gc.collect()
    gc.disable()
    try:
        t0 = time.perf_counter()
        for ev in evs:
            round_trip(ev)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    finally:
        gc.enable()
    e2e_ms = evs[0][0].elapsed_time(evs[-1][2])
    up = [e[0].elapsed_time(e[1]) for e in evs]
    sd = [e[1].elapsed_time(e[2]) for e in evs]
    e2e_val = cells * e2e_steps / (max(e2e_ms / 1e3, wall)) / 1e6
    nbytes = n_state * 8
    # the link on its own: one plain copy each way of the same bytes
    dev = torch.empty(n_state, dtype=torch.float64, device="cuda")
    link = {}
    for name, fn in (("h2d", lambda: dev.copy_(host, non_blocking=True)),
                     ("d2h", lambda: host.copy_(dev, non_blocking=True))):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        link[name] = a.elapsed_time(b)
    del dev
    # the same round trip with plain copies: copy in, full step, copy out
    seq = []
    import os as _os
    _os.environ["FST_NO_FUSED_UPLOAD"] = "1"
    try:
        for _ in range(3):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            assert L.fst_set_state(s._ctx, ptr, n_state) == 0
            assert L.fst_rk_step(s._ctx, 1) == 0
            assert L.fst_get_state(s._ctx, ptr, n_state) == 0
            b.record(stream)
            torch.cuda.synchronize()
            seq.append(a.elapsed_time(b))
    finally:
        del _os.environ["FST_NO_FUSED_UPLOAD"]
    e2e_detail = {"timed_steps": e2e_steps, "untimed_round_trips": 1,
                  "calls": "fst_set_state + fst_rk_step_get_state, page-locked host buffer",
                  "upload_ms_median": statistics.median(up),
                  "step_and_download_ms_median": statistics.median(sd),
                  "link_h2d_ms": link["h2d"], "link_h2d_gbs": nbytes / (link["h2d"] / 1e3) / 1e9,
                  "link_d2h_ms": link["d2h"], "link_d2h_gbs": nbytes / (link["d2h"] / 1e3) / 1e9,
                  "device_step_ms": ms / steps,
                  "plain_copies_round_trip_ms_median": statistics.median(seq),
                  "round_trip_ms_median": statistics.median([u + v for u, v in zip(up, sd)]),
                  "round_trip_ms": [round(e[0].elapsed_time(e[2]), 3) for e in evs],
                  "upload_ms": [round(x, 3) for x in up],
                  "step_and_download_ms": [round(x, 3) for x in sd],
                  "median_rate": cells / (statistics.median(
                      [u + v for u, v in zip(up, sd)]) / 1e3) / 1e6,
                  "wall_s": wall, "host_buffer": "pinned (cudaHostAlloc via torch)",
                  "python_gc": "disabled in the timed loop"}
    s.close()
    return U_final, {
        "value": value, "ms_per_step": ms / steps, "gpu_launches": launches, "hybrid": hybrid_info,
        "kernel_ms": {k: {"launches": v[0], "total_ms": v[1]} for k, v in kt.items()},
        "roofline": roof, "clocks": clk.summary(), "finite": finite,
        "e2e": {"value": e2e_val, "unit": "Mcell-steps/s", "h2d_bytes_per_step": n_state * 8,
                "d2h_bytes_per_step": n_state * 8, "steps": e2e_steps, **e2e_detail},
    }


def run_batch2d(steps, warmup, ncases=64):
    """The batched 2D ensemble (64 RT cases, n log-uniform in [128, 1024]):
    aggregate Mcell-steps/s with one persistent launch per stage under CUDA
    graph replay, against the same cases stepped one context at a time."""
    import torch
    from fiesta_gb300.batch import Batch, rt_ensemble
    from fiesta_gb300.solver import Solver
    cfgs, states = rt_ensemble(ncases=ncases)
    cells = sum(c.nci * c.ncj for c in cfgs)
    b = Batch(cfgs)
    for c, U in enumerate(states):
        b.set_state(c, U)
    # the tuner times every candidate in this run (force): its best and worst
    # times go on the bench line
    tune_path = os.path.join(ROOT, "fiesta_gb300", "tune_batch2d.json")
    shape = b.tune(tune_path, force=True)
    b.rk_step(warmup)
    b.synchronize()
    st = torch.cuda.ExternalStream(b.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    b.rk_step(steps)
    e1.record(st)
    b.synchronize()
    ms = e0.elapsed_time(e1) / steps
    info = b.info()
    b.close()
    # one context (one set of launches) per case
    ctxs = []
    for cfg, U in zip(cfgs, states):
        s = Solver(cfg)
        s.set_state(U)
        ctxs.append(s)
    stream = torch.cuda.current_stream()
    for s in ctxs:
        s.set_stream(stream.cuda_stream)
    for _ in range(warmup):
        for s in ctxs:
            s.rk_step(1)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        for s in ctxs:
            s.rk_step(1)
    e1.record(stream)
    torch.cuda.synchronize()
    ms1 = e0.elapsed_time(e1) / steps
    for s in ctxs:
        s.close()
    return {"value": cells / (ms / 1e3) / 1e6, "unit": "Mcell-steps/s", "ms_per_step": ms,
            "one_launch_per_case": cells / (ms1 / 1e3) / 1e6, "ms_per_step_per_case_launches": ms1,
            "ncases": ncases, "interior_cells": cells,
            "tile": {"width": shape[0], "height": shape[1], "blocks_per_sm": shape[2],
                     "max_blocks_per_sm": info["max_blocks_per_sm"]},
            "autotune": {"candidates": info["tune_candidates"],
                         "best_ms_per_step": info["tune_best_ms"],
                         "worst_ms_per_step": info["tune_worst_ms"],
                         "gain_over_worst": info["tune_worst_ms"] / info["tune_best_ms"],
                         "searched": "tile width {16,32,64} x height {4,8,16} (<=512 threads) x "
                                     "blocks/SM {m, 3m/4, m/2, m/4} (m = occupancy limit)"},
            "persistent_blocks": info["persistent_blocks"],
            "launches_per_step": info["launches_per_step"],
            "workload": "64 2D RT cases, n log-uniform in [128,1024], 2 species, viscous, "
                        "C-equation, buoyancy; mixed precision; CUDA graph per step"}


def gen3d_cfg(n, dt, mode=0):
    from fiesta_gb300 import abi
    return abi.make_config(3, (n, n, n), dx=(1.0, 1.0, 1.0), dt=dt, species=SPECIES,
                           grid_type=abi.GRID_GENERALIZED, mode=mode)


def gen3d_state(cfg, L):
    """The mixing case on a wavy grid of side L: interior from the seeded
    generator, ghosts filled once by outflow mirrors (the generalized module
    never fills them), and dt from the largest contravariant speed."""
    from fiesta_gb300 import abi
    from fiesta_gb300.grids import wavy_box
    from fiesta_gb300.solver import initial_conditions
    U0 = initial_conditions(cfg, abi.IC_MIXING_3D, SEED, **IC_KW)
    X = wavy_box(cfg, amp=0.25, L=L)
    S = max_wave_speed(cfg, U0) * cfg.nci / L  # |u|+c in cells per second
    return U0, X, 0.4 / S


def run_gen3d(n, steps, warmup, peak_gbs, peak_kind, mode=0):
    """The generalized-grid module (gen3d_func::compute) on a wavy 1 m box,
    plain FP64 (mode 0) or mixed (mode 1): Mcell-steps/s and the dominant
    kernel's roofline; returns the final state as well."""
    import torch
    from fiesta_gb300.solver import Solver
    cfg = gen3d_cfg(n, 1.0, mode)
    U0, X, dt = gen3d_state(cfg, 1.0)
    cfg.dt = dt
    s = Solver(cfg)
    stream = torch.cuda.current_stream()
    s.set_stream(stream.cuda_stream)
    s.set_state(U0)
    s.apply_bcs()
    s.set_grid(X)
    for _ in range(warmup):
        s.rk_step(1)
    torch.cuda.synchronize()
    l0 = s.stats()["kernel_launches"]
    s.set_profiling(True)
    s.kernel_times()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        s.rk_step(1)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    kt = s.kernel_times()
    s.set_profiling(False)
    launches = s.stats()["kernel_launches"] - l0
    finite = s.check_finite()
    U = s.get_state()
    s.close()
    top = max(kt.items(), key=lambda kv: kv[1][1])
    name, (nl, tot) = top
    b = algorithmic_bytes(name, cfg)
    ach = b / (tot / nl / 1e3) / 1e9 if b else None
    form = ("plain FP64 (bit-identical to the reference)" if mode == 0
            else "mixed precision (FP32 fluxes, FP64 state and pressure recovery)")
    return U, {"value": n ** 3 * steps / (ms / 1e3) / 1e6, "unit": "Mcell-steps/s",
               "ms_per_step": ms / steps, "gpu_launches": launches, "finite": finite,
               "dtype": "f64" if mode == 0 else "f32+f64",
               "workload": f"gen3d_func::compute on a wavy {n}^3 grid, 5 species, {form}",
               "kernel_ms": {k: {"launches": v[0], "total_ms": v[1]} for k, v in kt.items()},
               "roofline": {"bound": "fp64" if mode == 0 else "hbm", "kernel": name,
                            "achieved_hbm_gbs": ach, "peak_hbm_gbs": peak_gbs,
                            "hbm_frac": ach / peak_gbs if ach else None, "peak_source": peak_kind,
                            "algorithmic_bytes_per_launch": b, "avg_launch_ms": tot / nl}}


def cpu_sample_gen3d(n_sample=256, steps=1):
    """The CPU oracle's generalized 3D step on a bounded sample."""
    from oracle.oracle import Oracle
    cores = os.cpu_count() or 1
    Oracle.set_threads(cores)
    cfg = gen3d_cfg(n_sample, 1.0)
    U0, X, dt = gen3d_state(cfg, 1.0)
    cfg.dt = dt
    o = Oracle(cfg)
    o.set_state(U0)
    o.apply_bcs()
    o.set_grid(X)
    t0 = time.perf_counter()
    o.rk_step(steps)
    el = time.perf_counter() - t0
    return {"value": n_sample ** 3 * steps / el / 1e6, "unit": "Mcell-steps/s", "cores": cores,
            "kind": "port", "sample": f"{steps} step(s) at {n_sample}^3 ({el:.1f} s)"}


def run_aux(n, U0, dt, peak_gbs, peak_kind, reps=3, cpu=True):
    """The postStep work beside the step, on the headline mixed context:
    secondary variables (rho, p, T, velocity over all cells), the status
    min/max reduction, and the noise filter (momenta, one sweep); device time
    per call from the kernels' CUDA events, against the HBM roof, and the CPU
    oracle on the same calls."""
    import torch
    from fiesta_gb300.solver import Solver
    cfg = make_cfg(n, MODES["mixed"], dt)
    s = Solver(cfg)
    s.set_stream(torch.cuda.current_stream().cuda_stream)
    s.set_state(U0)
    s.secondary()
    s.set_profiling(True)
    s.kernel_times()
    for _ in range(reps):
        s.secondary()
        s.status(secondary=False)
        s.noise_filter(1e-3, 0.1, 0.5, 1, 1)
    kt = s.kernel_times()
    # the noise filter as it runs unprofiled: its sweeps replay as one CUDA
    # graph, timed as a whole with events on the library's stream
    s.set_profiling(False)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.noise_filter(1e-3, 0.1, 0.5, 1, 1)  # captures the graph
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        s.noise_filter(1e-3, 0.1, 0.5, 1, 1)
    e1.record(stream)
    torch.cuda.synchronize()
    noise_ms = e0.elapsed_time(e1) / reps
    s.close()
    allc = (n + 6) ** 3
    inner = n ** 3
    nv, nvt = 4 + cfg.ns, 4 + cfg.ns + 5
    noise_kernels = {k: v[1] / reps for k, v in kt.items() if k.startswith("noise")}
    rows = {
        # reads the state's nv fields, writes rho, p, u, v, w, T (FP64)
        "secondary": (kt.get("secondary", (0, 0.0))[1] / reps, allc * 8 * (nv + 6)),
        # reads the nvt state fields over the interior
        "status": (kt.get("status", (0, 0.0))[1] / reps, inner * 8 * nvt),
        # compulsory: the cutoff's C variable (maximum), the three momenta once,
        # the indicator written; a sweep that changes no cell moves nothing more
        "noise_filter": (noise_ms, inner * (8 + 3 * 8 + 4)),
    }
    out = {}
    for k, (ms, b) in rows.items():
        ach = b / (ms / 1e3) / 1e9 if ms > 0 else None
        out[k] = {"ms_per_call": ms, "algorithmic_bytes": b, "achieved_gbs": ach,
                  "hbm_frac": ach / peak_gbs if ach else None, "peak_source": peak_kind}
    out["noise_filter"]["launches_per_call"] = sum(v[0] for k, v in kt.items()
                                                   if k.startswith("noise")) // reps
    out["noise_filter"]["profiled_ms_per_kernel"] = noise_kernels
    out["noise_filter"]["timing"] = ("whole calls, CUDA events (sweeps replayed as a CUDA graph); "
                                     "profiled_ms_per_kernel: the same calls launched one by one")
    if cpu:  # the oracle on the same calls (OpenMP; the noise filter's sweep is serial)
        from oracle.oracle import Oracle
        cores = os.cpu_count() or 1
        Oracle.set_threads(cores)
        o = Oracle(make_cfg(n, 0, dt))
        o.set_state(U0)
        t0 = time.perf_counter()
        o.secondary()
        t1 = time.perf_counter()
        o.noise_filter(1e-3, 0.1, 0.5, 1, 1)
        t2 = time.perf_counter()
        out["cpu_oracle"] = {"cores": cores, "secondary_ms": (t1 - t0) * 1e3,
                             "noise_filter_ms": (t2 - t1) * 1e3,
                             "note": "secondary includes its host repack; the noise "
                                     "filter's removal sweep is serial by definition"}
    out["workload"] = f"{n}^3 mixing case, mixed context; noise filter mode 1 (momenta), nt = 1"
    return out


def accuracy_report(cfg, U0, finals, nsteps):
    """rel-L2 per state field (conserved and C-equation) over the interior,
    after the same steps:
    mixed and hybrid against the plain FP64 path (bit-identical to the
    reference's FP64 arithmetic), and hybrid against mixed (full WENO).
    Fields that start at zero are compared by their increment."""
    names = ["x-momentum", "y-momentum", "z-momentum", "energy"] + \
            [f"species{s}" for s in range(cfg.ns)] + ["C", "C_hat", "C_1", "C_2", "C_3"]
    ng = cfg.ng

    def I(A, v):
        return A[ng:-ng, ng:-ng, ng:-ng, v]

    def rel(a, b):
        d = np.linalg.norm((a - b).ravel())
        nb = np.linalg.norm(b.ravel())
        return float(d / nb) if nb > 0 else float(d)

    out = {"steps": nsteps}
    pairs = [(m, "plain") for m in ("mixed", "hybrid") if m in finals and "plain" in finals]
    if "plain_perturbed" in finals and "plain" in finals:
        # the condition spread: how far the FP64 path itself moves when its
        # initial state is perturbed by COND_EPS (relative, seeded)
        pairs.insert(0, ("plain_perturbed", "plain"))
    if "hybrid" in finals and "mixed" in finals:
        pairs.append(("hybrid", "mixed"))
    for a_, b_ in pairs:
        rows = {}
        for v, name in enumerate(names):
            z = I(U0, v)
            if np.abs(z).max() > 0:
                rows[name] = rel(I(finals[a_], v), I(finals[b_], v))
            else:
                rows[name + " (increment)"] = rel(I(finals[a_], v) - z, I(finals[b_], v) - z)
        out[f"{a_}_vs_{b_}"] = rows
    return out


COND_EPS = 1e-8      # relative perturbation of the initial state (condition spread)
COND_FACTOR = 10.0   # a field passes at max(1e-5, COND_FACTOR * its condition spread)


def perturbed(U0, eps=COND_EPS, seed=1):
    rng = np.random.default_rng(seed)
    U = U0.copy()
    nz = np.abs(U0) > 0
    U[nz] *= 1 + eps * rng.standard_normal(int(nz.sum()))
    return np.asfortranarray(U)


def plain_final(n, U, dt, nsteps):
    """State of the plain FP64 path (bit-identical to the reference's
    arithmetic) after nsteps from U."""
    from fiesta_gb300.solver import Solver
    s = Solver(make_cfg(n, MODES["plain"], dt))
    s.set_state(U)
    s.rk_step(nsteps)
    out = s.get_state()
    s.close()
    return out


def cpu_sample(n_sample=128, steps=3, kind=None):
    """The reference's FP64 step on the host cores, on a bounded sample of
    the same workload: its own sources (src/cart3d.cpp, src/rk.cpp and the
    kernel headers, built by oracle/ref_build.sh into oracle/_ref) where that
    library exists (kind "reference"), else the oracle restatement (kind
    "port"); OpenMP on every host core.  The seeded initial state comes from
    the numpy restatement of the generator (oracle/ics.py), so this leg loads
    no product library.  Returns the median per-step rate."""
    from oracle.ics import mixing_3d
    from oracle.oracle import Oracle, Reference
    if kind is None:
        kind = "reference" if Reference.available() else "port"
    cores = os.cpu_count() or 1
    cfg = make_cfg(n_sample, 0, 1.0)
    U0 = mixing_3d(cfg, SEED, **IC_KW)
    cfg.dt = bench_dt(cfg, U0)
    if kind == "reference":
        o = Reference(cfg)
    else:
        Oracle.set_threads(cores)
        o = Oracle(cfg)
    o.set_state(U0)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        o.rk_step(1)
        times.append(time.perf_counter() - t0)
    del o
    per = statistics.median(times)
    what = ("the reference's own sources (src/cart3d.cpp, src/rk.cpp, kernel headers) "
            "built by oracle/ref_build.sh" if kind == "reference"
            else "the CPU oracle restatement of the reference's FP64 path")
    return {"value": n_sample ** 3 / per / 1e6, "unit": "Mcell-steps/s", "cores": cores,
            "kind": kind,
            "sample": f"median of {steps} step(s) of the same case at {n_sample}^3, {what}, "
                      f"OpenMP on {cores} threads ({per:.2f} s per step)"}


def replica_value(ms, n, world, device):
    """Whole-job Mcell-steps/s of `world` replicas of an n^3 case: every rank
    runs the whole case, the slowest rank's ms per step sets the pace."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    return world * (n ** 3) / (ms / 1e3) / 1e6, ms


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--modes", default="plain,mixed,hybrid")
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--e2e-steps", type=int, default=30)
    # the CPU legs: a bounded sample of the same case for the baseline beside
    # the GPU line, the full case for the reference arm (the reference's own
    # build runs ~6x slower than the oracle restatement)
    ap.add_argument("--cpu-sample", type=int, default=128)
    ap.add_argument("--ref-sample", type=int, default=256)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-gen", action="store_true")
    ap.add_argument("--no-aux", action="store_true")
    a = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    a.warmup = max(a.warmup, 3)

    if a.impl == "reference":
        # The reference has no GPU path here (its Kokkos CUDA build is not
        # available); its own FP64 CPU build is timed on the host cores,
        # with the oracle restatement beside it as a second figure.
        if rank != 0:
            return
        t0 = time.perf_counter()
        cb = cpu_sample(a.ref_sample, max(1, min(a.steps, 2)))
        val = cb["value"]
        line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "Mcell-steps/s",
                "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
                "ms_per_step": (a.size ** 3) / (val * 1e6) * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded generator: 8 Gaussian pressure kernels, 5 species)",
                "config": {"workload": workload(a.size), "grid": [a.size] * 3, "species": 5,
                           "nvt": 14, "mode": "plain", "sample_grid": [a.ref_sample] * 3},
                "cpu_baseline": cb,
                "e2e": {"value": val, "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        if cb["kind"] == "reference":
            line["restatement"] = cpu_sample(a.ref_sample, max(1, min(a.steps, 2)), kind="port")
        line["wall_s"] = time.perf_counter() - t0
        print(json.dumps(line))
        return

    import torch
    from fiesta_gb300 import abi
    from fiesta_gb300.solver import initial_conditions
    if world > 1:
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        import torch.distributed as dist
        dist.init_process_group("nccl")
    peak, peak_kind = load_peaks()
    n = a.size
    cfg0 = make_cfg(n, 0, 1.0)
    U0 = initial_conditions(cfg0, abi.IC_MIXING_3D, SEED, **IC_KW)
    dt = bench_dt(cfg0, U0)
    modes = [m.strip() for m in a.modes.split(",") if m.strip()]
    results, finals = {}, {}
    for m in modes:
        finals[m], results[m] = run_gpu_mode(m, n, a.steps, a.warmup, U0, dt, peak, peak_kind,
                                             a.e2e_steps)
    if "plain" in finals and len(modes) > 1:
        finals["plain_perturbed"] = plain_final(n, perturbed(U0), dt, a.warmup + a.steps)
    accuracy = accuracy_report(make_cfg(n, 0, dt), U0, finals, a.warmup + a.steps)
    del finals
    # headline: the fastest mode whose every state field (conserved and
    # C-equation) is within max(1e-5, COND_FACTOR x the field's condition
    # spread) of the FP64 path, which is bit-identical to the reference's
    # arithmetic
    spread = (accuracy or {}).get("plain_perturbed_vs_plain", {})

    def within(m):
        if m == "plain":
            return True
        rows = (accuracy or {}).get(f"{m}_vs_plain", {})
        return bool(rows) and all(e <= max(1e-5, COND_FACTOR * spread.get(k, 0.0))
                                  for k, e in rows.items())
    ok = [m for m in modes if within(m)]
    unchecked = not ok  # a run without the plain mode has nothing to judge against
    head = max(ok or modes, key=lambda m: results[m]["value"])
    # replicas only: each rank runs the whole case; whole-job value sums ranks
    r = results[head]
    value, ms = r["value"], r["ms_per_step"]
    if world > 1:
        value, ms = replica_value(ms, n, world, "cuda")
    if rank != 0:
        return
    batch = None if a.no_batch else run_batch2d(a.steps, a.warmup)
    gen3d = None
    if not a.no_gen:
        Up, gen3d = run_gen3d(n, a.steps, a.warmup, peak, peak_kind, 0)
        Um, gen3d["mixed"] = run_gen3d(n, a.steps, a.warmup, peak, peak_kind, 1)
        gcfg = gen3d_cfg(n, 1.0)
        ng, nsteps = gcfg.ng, a.warmup + a.steps
        G0, _, _ = gen3d_state(gcfg, 1.0)
        rows = {}
        for v in range(Up.shape[3]):  # momenta by their increments (they start at zero)
            z = G0[ng:-ng, ng:-ng, ng:-ng, v] if v < 3 else 0.0
            pa, ma = Up[ng:-ng, ng:-ng, ng:-ng, v] - z, Um[ng:-ng, ng:-ng, ng:-ng, v] - z
            nb = np.linalg.norm(pa.ravel())
            rows[v] = float(np.linalg.norm((ma - pa).ravel()) / nb) if nb > 0 else 0.0
        gen3d["mixed"]["rel_l2_vs_plain_after_steps"] = {"steps": nsteps, "max": max(rows.values()),
                                                          "per_variable": rows}
        del Up, Um, G0
        if not a.no_cpu:
            gen3d["cpu_baseline"] = cpu_sample_gen3d(min(n, a.cpu_sample))
    aux = None if a.no_aux else run_aux(n, U0, dt, peak, peak_kind, cpu=not a.no_cpu)
    cpu = None if a.no_cpu else cpu_sample(a.cpu_sample, 2)
    line = {
        "metric": METRIC, "value": value, "unit": "Mcell-steps/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if head == "plain" else "f32+f64",
        "data": "synthetic (seeded compiled IC generator: 8 Gaussian pressure kernels, 5 species)",
        "config": {"workload": workload(n), "grid": [n] * 3, "species": 5, "nvt": 14,
                   "mode": head, "headline_rule": "fastest mode with every state field "
                   "(conserved and C-equation) within rel-L2 max(1e-5, 10 x its condition "
                   "spread) of the FP64 path after warmup+steps steps; the condition spread is "
                   "the FP64 path's own change from a 1e-8 relative perturbation of the "
                   "initial state, the size of the mixed path's conserved-field error "
                   "(accuracy.plain_perturbed_vs_plain)"
                   + ("; not applied in this run: the plain mode did not run" if unchecked
                      else ""),
                   "dt": dt, "l2": f"state {(n + 6) ** 3 * 14 * 8 / 1e9:.2f} GB "
                   f"{'>' if (n + 6) ** 3 * 14 * 8 > 129e6 else '<'} L2 (129 MB)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": r["roofline"],
        # whole-step figure: the compulsory FP64 state traffic of a fused
        # two-stage RK step, 5 * nvt * 8 bytes per interior cell-step
        "roofline_step": {"bytes_per_cell_step": 5 * 14 * 8,
                          "achieved": value * 1e6 * 5 * 14 * 8 / 1e9, "unit": "GB/s",
                          "peak": peak, "frac": value * 1e6 * 5 * 14 * 8 / 1e9 / peak,
                          "peak_source": peak_kind},
        "cpu_baseline": cpu, "clocks": r["clocks"],
        "e2e": r["e2e"], "gpu_launches": r["gpu_launches"],
        "modes": {m: {k: v for k, v in results[m].items() if k not in ("clocks",)} for m in modes},
        "batch2d": batch,
        "gen3d": gen3d,
        "aux": aux,
        "accuracy": accuracy,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
