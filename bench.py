#!/usr/bin/env python
"""Benchmark of the GB300 AMR hot path: cell-updates/s.

Headline workload (one bench step = one complete run of it): the batched
form, FP32.  512 independent 2D linear-advection AMR instances held in one
forest (one tree object; each instance is its own periodic unit square):
16x16-cell patches + 1 ghost layer, seeded depth caps 2-6 (each instance is
refined to its cap and held there, min = max level, so leaf counts are
16-4096 and ~560k patches in total), seeded velocities in [-1,1]^2, two
seeded Gaussian bumps per instance (sigma 0.02-0.06, amplitude 0.5-2), CFL
0.4, gradient criterion 0.05 / 0.01 and re-mesh every 10 steps, 1000 steps.
Each re-mesh interval is one CUDA graph replay (step coefficients, 10 update
steps, halo fill, flags, 2:1 closure, scan, emit, remap, neighbour rebuild);
the update kernel's launch shape is picked by the autotuner on first use.
cell-updates = sum over intervals of steps x leaves x 16^2, re-mesh time
included (the reference's definition,
benchmark/bench_fvm_solver_integration_active_amr.b.cpp:244-245, 258).

The same forest is run in FP64 (the plain drop-in arithmetic) for the
FP32/FP64 throughput ratio and the relative L2 error of the FP32 state.  The
plain FP64 drop-in on the single-tree active-AMR workload (2000 steps, max
level 5) is reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`value` times K runs with the initial state already in HBM; `e2e` times K runs
through the C ABI with the initial state copied from pinned host memory and
the final state copied back inside the timed region.  L2 is flushed (256 MiB
write) before every timed run, outside the timed interval.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "gpu-amr_gb300"))
sys.path.insert(0, str(REPO))

METRIC = "cell-updates/s FP32-batched vs FP64-plain at stated L2 err; adjoint/forward cost"
UNIT = "cell-updates/s"

BATCHED = dict(
    instances=512, n=16, halo=1, depth=6, cap_lo=2, cap_hi=6, steps=1000, remesh=10, cfl=0.4, rthr=0.05, cthr=0.01,
    seed=3, bumps=2, sigma=(0.02, 0.06), amp=(0.5, 2.0),
)
BATCHED_NAME = ("batched, static caps: 512 independent 2D advection AMR instances in one forest, 16x16 patches + 1 ghost, "
                "seeded depth caps 2-6 (refined to the cap and held: min = max level), seeded velocities in "
                "[-1,1]^2, 2 seeded Gaussian bumps each, grad criterion 0.05/0.01, re-mesh every 10 steps "
                "(one CUDA graph replay per interval), CFL 0.4, 1000 steps, FP32 state")

WORKLOAD = dict(
    rank=2, n=16, halo=1, depth=7, init_levels=2, steps=2000, remesh=10, velocity=(1.0, 0.5), cfl=0.4,
    rthr=0.05, cthr=0.01, min_level=1, max_level=5, bump_seed=2, noise=1e-3, noise_seed=2,
)
WORKLOAD_NAME = ("2D linear advection, active AMR, FP64 plain: 16x16 patches + 1 ghost, max level 5, "
                 "grad criterion 0.05/0.01, re-mesh every 10 steps, 2 seeded Gaussian bumps, v=(1,0.5), "
                 "periodic, CFL 0.4, 2000 steps")


def measured_peaks():
    try:
        return json.loads((REPO / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi sampling during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.idx = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ GPU arm
def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


# ------------------------------------------------------------ batched form
def batched_instances():
    """Seeded per-instance parameters: depth cap, velocity, Gaussian bumps
    (centre x, centre y, sigma, amplitude per bump)."""
    B = BATCHED
    rng = np.random.default_rng(B["seed"])
    K = B["instances"]
    caps = rng.integers(B["cap_lo"], B["cap_hi"] + 1, K).astype(np.int32)
    vel = rng.uniform(-1.0, 1.0, (K, 2))
    bumps = np.zeros((K, B["bumps"], 4))
    bumps[..., 0:2] = rng.uniform(0.15, 0.85, (K, B["bumps"], 2))
    bumps[..., 2] = rng.uniform(*B["sigma"], (K, B["bumps"]))
    bumps[..., 3] = rng.uniform(*B["amp"], (K, B["bumps"]))
    return caps, vel, bumps


def batched_ic(torch, ids, bumps, dev):
    """Padded FP64 initial state on the device: per leaf, the sum of its
    instance's Gaussian bumps at the cell centres (physics_system::cell_coord
    geometry on the unit square), ghosts zero."""
    B = BATCHED
    n, h, depth = B["n"], B["halo"], B["depth"]
    k = torch.from_numpy(np.asarray(ids, np.uint64).view(np.int64)).to(dev)
    level = (k & 63).to(torch.float64)
    m = (k >> 6) & ((1 << (2 * depth)) - 1)
    inst = k >> (6 + 2 * depth)
    x = torch.zeros_like(m)
    y = torch.zeros_like(m)
    for b in range(depth):
        x |= ((m >> (2 * b)) & 1) << b
        y |= ((m >> (2 * b + 1)) & 1) << b
    maxc = float(1 << depth)
    cs = (torch.pow(2.0, depth - level) / maxc / n)[:, None, None]
    i = torch.arange(n, device=dev, dtype=torch.float64)
    cx = (x.to(torch.float64) / maxc)[:, None, None] + i[None, None, :] * cs + 0.5 * cs
    cy = (y.to(torch.float64) / maxc)[:, None, None] + i[None, :, None] * cs + 0.5 * cs
    bp = torch.from_numpy(bumps).to(dev)[inst]  # (P, nb, 4)
    val = torch.zeros((k.shape[0], n, n), dtype=torch.float64, device=dev)
    for j in range(bp.shape[1]):
        c = bp[:, j]
        r2 = (cx - c[:, 0, None, None]) ** 2 + (cy - c[:, 1, None, None]) ** 2
        val += c[:, 3, None, None] * torch.exp(-r2 / (2.0 * c[:, 2, None, None] ** 2))
    out = torch.zeros((k.shape[0], n + 2 * h, n + 2 * h), dtype=torch.float64, device=dev)
    out[:, h:n + h, h:n + h] = val
    return out, inst


def make_forest(A, dtype, stream, caps, vel, bounds=None):
    """The batched forest refined to its caps; level bounds per instance
    (default: held at the cap)."""
    B = BATCHED
    K = B["instances"]
    cap = int(np.sum(4 ** caps.astype(np.int64))) + 1024
    f = A.Tree(2, B["n"], B["halo"], B["depth"], capacity=cap, dtype=dtype, stream=stream.cuda_stream, instances=K)
    f.refine_to_levels(caps)
    f.set_instance_params(velocity=vel, level_bounds=np.stack([caps, caps], 1) if bounds is None else bounds)
    return f


def run_forest(f):
    B = BATCHED
    return f.run(B["steps"], B["remesh"], None, B["cfl"], "grad", B["rthr"], B["cthr"], instance_params=True)


def time_runs(torch, stream, world, k, setup, body, flush, clocks=None):
    """k timed runs: setup + L2 flush outside, CUDA events around body on the
    forest's stream.  Returns (ms, launches, stats)."""
    import amr_gb300 as A

    total_ms, launches, stats = 0.0, 0, []
    if clocks:
        clocks.start()
    for _ in range(k):
        setup()
        flush.zero_()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        l0 = A.launch_count()
        ev0, ev1 = _events(torch)
        ev0.record(stream)
        stats.append(body())
        ev1.record(stream)
        torch.cuda.synchronize()
        launches += A.launch_count() - l0
        total_ms += ev0.elapsed_time(ev1)
    info = clocks.stop() if clocks else None
    return total_ms, launches, stats, info


# runs of the end-to-end pipeline: the first upload and the last download
# are not hidden behind a run, so more runs amortise them
E2E_RUNS = 8


def copy_rates(torch, stream, dev, host_in, host_out):
    """GB/s of one pinned host -> device and one device -> host copy of the
    state, each timed alone with CUDA events on the forest's stream."""
    out = []
    with torch.cuda.stream(stream):
        for src, dst in ((host_in, dev), (dev, host_out)):
            dst.copy_(src, non_blocking=True)
            torch.cuda.synchronize()
            e0, e1 = _events(torch)
            e0.record(stream)
            dst.copy_(src, non_blocking=True)
            e1.record(stream)
            torch.cuda.synchronize()
            out.append(src.numel() * src.element_size() / (e0.elapsed_time(e1) * 1e-3) / 1e9)
    return out


def e2e_pipeline(torch, stream, f, P, like, host_in, host_out, K, warmup, world):
    """K complete runs of forest f, each fed from pinned host memory and read
    back to it, copies overlapped with the runs on a second stream.  Returns
    (ms of the K runs, cell updates); warm-up runs first."""
    copy = torch.cuda.Stream()
    st_in = [torch.empty_like(like) for _ in range(2)]
    st_out = [torch.empty_like(like) for _ in range(2)]
    ev = {k: [torch.cuda.Event() for _ in range(2)] for k in ("in", "used", "res", "out")}

    def pipeline(n):
        e0, e1 = _events(torch)
        e0.record(stream)
        copy.wait_event(e0)
        with torch.cuda.stream(copy):
            st_in[0].copy_(host_in, non_blocking=True)
            ev["in"][0].record(copy)
        cells = 0
        for k in range(n):
            b = k % 2
            stream.wait_event(ev["in"][b])
            f.load_state_device(st_in[b].data_ptr(), P)
            ev["used"][b].record(stream)
            if k + 1 < n:  # the next run's input, into the other staging buffer
                nb = (k + 1) % 2
                with torch.cuda.stream(copy):
                    if k >= 1:
                        copy.wait_event(ev["used"][nb])
                    st_in[nb].copy_(host_in, non_blocking=True)
                    ev["in"][nb].record(copy)
            cells += run_forest(f)["cell_updates"]
            if k >= 2:
                stream.wait_event(ev["out"][b])  # run k - 2's download has read st_out[b]
            f.download_state_device(st_out[b].data_ptr(), P)
            ev["res"][b].record(stream)
            with torch.cuda.stream(copy):
                copy.wait_event(ev["res"][b])
                host_out[b].copy_(st_out[b], non_blocking=True)
                ev["out"][b].record(copy)
        stream.wait_stream(copy)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), cells

    pipeline(max(1, warmup))  # the host buffers' first transfers are not part of a step
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    return pipeline(K)


def batched_arm(args, torch, A, dev, stream, flush, world):
    B = BATCHED
    caps, vel, bumps = batched_instances()
    f32 = make_forest(A, A.F32, stream, caps, vel)
    ids = f32.ids()
    P = len(ids)
    ic64, inst = batched_ic(torch, ids, bumps, dev)
    ic32 = ic64.to(torch.float32).contiguous()
    ic32_host = ic32.cpu().pin_memory()
    out32_host = torch.empty_like(ic32_host).pin_memory()

    def load32():
        f32.load_state_device(ic32.data_ptr(), P)

    for _ in range(args.warmup):
        load32()
        run_forest(f32)
    ms, launches, stats, clock_info = time_runs(torch, stream, world, args.steps, load32, lambda: run_forest(f32),
                                                flush, ClockSampler(dev))
    tuned = f32.step_config()
    cells = sum(s["cell_updates"] for s in stats)
    assert all(s["leaves_min"] == s["leaves_max"] == P for s in stats)
    fin32 = torch.empty_like(ic32)
    f32.download_state_device(fin32.data_ptr(), P)

    # end to end, K runs: each run's initial state comes from pinned host
    # memory and its final state goes back to pinned host memory; the copies
    # run on a second stream, the upload of run k + 1 and the download of run
    # k - 1 beside run k (two device staging buffers each way)
    out32_host2 = torch.empty_like(ic32_host).pin_memory()
    e2e_runs = max(args.steps, E2E_RUNS)
    e2e_ms, e2e_cells = e2e_pipeline(torch, stream, f32, P, ic32, ic32_host, [out32_host, out32_host2], e2e_runs,
                                     args.warmup, world)
    # the host link alone: one state upload and one download, timed apart
    h2d_gbs, d2h_gbs = copy_rates(torch, stream, ic32, ic32_host, out32_host)

    # the update kernel alone: CUDA events around each launch on the forest's
    # stream, in a complete run whose intervals are issued directly instead of
    # replayed from the graph (same kernels, same order)
    load32()
    f32.set_timing(True)
    run_forest(f32)
    k_ms, k_launches, k_cells = f32.get_timing()
    if k_launches == 0:  # the fused interval kernel is off: time the multi-step passes
        load32()
        f32.advance(50, None, B["cfl"])
        f32.finish_advance()
        k_ms, k_launches, k_cells = f32.get_timing()
    f32.set_timing(False)

    # FP64 plain arithmetic on the same forest
    f64 = make_forest(A, A.F64, stream, caps, vel)
    assert np.array_equal(f64.ids(), ids)

    def load64():
        f64.load_state_device(ic64.data_ptr(), P)

    load64()
    run_forest(f64)
    ms64, _, stats64, _ = time_runs(torch, stream, world, max(1, args.steps), load64, lambda: run_forest(f64), flush)
    cells64 = sum(s["cell_updates"] for s in stats64)
    fin64 = torch.empty_like(ic64)
    f64.download_state_device(fin64.data_ptr(), P)

    # parity sample: the CPU baseline's instances, the same number of steps,
    # from the same initial state, in FP64 and FP32 (compared in main())
    npar, spar = CPU_SAMPLE["instances"], CPU_SAMPLE["steps"]
    off = f32.instance_offsets()
    mask = np.uint64((1 << (6 + 2 * B["depth"])) - 1)
    parity = {"init": [ic64[off[i]:off[i + 1]].cpu().numpy() for i in range(npar)], "steps": spar}
    for key, f, ic in (("f64", f64, ic64), ("f32", f32, ic32)):
        f.load_state_device(ic.data_ptr(), P)
        f.run(spar, B["remesh"], None, B["cfl"], "grad", B["rthr"], B["cthr"], instance_params=True)
        fin = torch.empty_like(ic)
        f.download_state_device(fin.data_ptr(), P)
        o = f.instance_offsets()
        ids = f.ids()
        parity[key] = [(ids[o[i]:o[i + 1]] & mask, fin[o[i]:o[i + 1]].double().cpu().numpy()) for i in range(npar)]
    n, h = B["n"], B["halo"]
    a = fin32[:, h:n + h, h:n + h].to(torch.float64)
    b = fin64[:, h:n + h, h:n + h]
    rel = float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
    K = B["instances"]
    num = torch.zeros(K, dtype=torch.float64, device=dev).index_add_(0, inst, ((a - b) ** 2).sum((1, 2)))
    den = torch.zeros(K, dtype=torch.float64, device=dev).index_add_(0, inst, (b ** 2).sum((1, 2)))
    rel_inst = float(torch.sqrt(num / den).max())
    ok = np.isfinite(rel) and rel <= 1e-5
    acc32, _ = f32.instance_time()
    f32.close()
    f64.close()

    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    # a launch reads and writes every interior cell once (FP32) and applies
    # `per_pass` updates to it (the whole ten-step interval on this forest)
    cells_per_launch = k_cells / k_launches if k_launches else 0
    per_pass = int(round(cells_per_launch / (P * B["n"] ** 2))) if k_launches else 1
    alg = 8.0 * P * B["n"] ** 2 * k_launches
    achieved = alg / (k_ms * 1e-3) / 1e9 if k_ms > 0 else None
    traffic = None
    kname = "k_run_interval2d" if per_pass == 10 else f"k_step2d_pass{per_pass}"
    prof = REPO / "profiles" / f"{kname}_fp32_forest.json"
    if prof.exists():
        try:
            per_patch = json.loads(prof.read_text()).get("dram_bytes_per_patch")
            traffic = per_patch * P if per_patch else None
        except Exception:
            traffic = None
    value = cells / (ms * 1e-3)
    value64 = cells64 / (ms64 * 1e-3)
    return {
        "value": value,
        "parity": parity,
        "ms": ms,
        "cells": cells,
        "e2e_ms": e2e_ms,
        "e2e_cells": e2e_cells,
        "launches": launches,
        "clocks": clock_info,
        "config": {
            "workload": BATCHED_NAME,
            "instances": K,
            "patches": P,
            "leaves_per_instance": {"min": int(4 ** caps.min()), "max": int(4 ** caps.max())},
            "cap_histogram": {str(c): int((caps == c).sum()) for c in range(B["cap_lo"], B["cap_hi"] + 1)},
            "step": "one complete 1000-step run (100 re-mesh intervals, one graph replay each) from the initial state",
            "l2": "flushed (256 MiB write) before every timed run, outside the timed interval; "
                  "the state (2 x 0.73 GB) exceeds L2 in any case",
            "sum_dt_instance0": float(acc32[0]),
            "driver": f"graph replays per run: {stats[0]['graph_intervals']} of {stats[0]['intervals']} intervals",
            "autotuned_update_kernel": {"warps_per_block": tuned[0], "copy_stages": tuned[1],
                                        "blocks": tuned[2] or "full residency"},
        },
        "e2e": {"value": e2e_cells / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(ic32_host.numel() * 4),
                "d2h_bytes_per_step": int(out32_host.numel() * 4), "runs": e2e_runs,
                "note": "each run uploads its initial state from pinned host memory and downloads its final state; "
                        "the copies of neighbouring runs overlap the run on a second stream",
                "host_link_gbs": {"h2d": h2d_gbs, "d2h": d2h_gbs}},
        "roofline": {
            "bound": "hbm",
            "kernel": ("k_run_interval2d<10,true> (the whole re-mesh interval, ten steps and the gradient flags, "
                       "in one pass over memory per 4x4-patch block: every relation of the forest is same-level)")
                      if per_pass == 10 else
                      (f"k_step2d_pass<float,16,1,W,S,{per_pass}> ({per_pass} steps per pass over memory: every "
                       f"relation of the forest is same-level)") if per_pass > 1 else "k_step2d<float,16,1,W,S>",
            "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": (achieved / hbm) if (achieved and hbm) else None,
            "traffic": traffic,
            "algorithmic_bytes_per_launch": alg / k_launches if k_launches else None,
            "cell_updates_per_pass": per_pass,
            "algorithmic_bytes_per_cell_update": 8 / per_pass,
            "per_cell_update_definition": {
                "achieved": (8.0 * k_cells / (k_ms * 1e-3) / 1e9) if k_ms > 0 else None,
                "frac": (8.0 * k_cells / (k_ms * 1e-3) / 1e9 / hbm) if (k_ms > 0 and hbm) else None,
                "note": "8 B (one FP32 read and write) per cell update, as if every step went through HBM; above 1 "
                        "because a launch applies ten steps to each cell it reads once"},
            "note": "achieved = one FP32 read + write of every interior cell per launch / CUDA-event launch time "
                    "(launches timed inside a complete run)",
            "launches": k_launches, "avg_launch_us": (k_ms * 1e3 / k_launches) if k_launches else None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured, burst copy)" if hbm else "missing",
        },
        "fp64_plain_same_workload": {
            "value": value64, "unit": UNIT, "ms_per_run": ms64 / max(1, args.steps),
            "ratio_fp32_batched_over_fp64": value / value64,
            "note": "the same forest, state and arithmetic in FP64 (the plain drop-in kernels)",
        },
        "precision": {
            "rel_l2_fp32_vs_fp64": rel, "max_instance_rel_l2": rel_inst, "bar": 1e-5, "within_bar": bool(ok),
            "reference": "FP64 run of the same forest on the GPU (the FP64 path equals the oracle within 1e-12)",
            "fp64_kept_for": "CFL step, coarse-fine restriction/prolongation means, gradient flags",
        },
    }


# ------------------------------------------------ batched form, adapting
ACTIVE_NAME = ("batched, adapting: the batched workload's 512 instances, each free to coarsen two levels below "
               "its cap and to refine back to it (level bounds (cap - 2, cap)), so the gradient flags re-mesh "
               "the forest every interval; 1000 steps, FP32 state")


def precision_history(A, torch, stream, caps, vel, bounds, ic32, ic64, reset, dev):
    """FP32 and FP64 runs of the adapting forest, one re-mesh interval per
    call; per instance the first interval after which its FP32 tree differs
    from its FP64 tree (none: the same tree after every re-mesh), and the
    final relative L2 of FP32 against FP64 per instance."""
    B = BATCHED
    f32 = make_forest(A, A.F32, stream, caps, vel, bounds)
    f64 = make_forest(A, A.F64, stream, caps, vel, bounds)
    reset(f32, ic32)
    reset(f64, ic64)
    K = len(caps)
    parted = np.full(K, -1, np.int64)
    nint = B["steps"] // B["remesh"]
    for k in range(nint):
        for f in (f32, f64):
            f.run(B["remesh"], B["remesh"], None, B["cfl"], "grad", B["rthr"], B["cthr"], instance_params=True)
        a, b = f32.ids(), f64.ids()
        oa, ob = f32.instance_offsets(), f64.instance_offsets()
        for i in np.nonzero(parted < 0)[0]:
            if not np.array_equal(a[oa[i]:oa[i + 1]], b[ob[i]:ob[i + 1]]):
                parted[i] = k
    n, h = B["n"], B["halo"]
    s32 = torch.empty((len(f32.ids()), n + 2, n + 2), dtype=torch.float32, device=dev)
    s64 = torch.empty((len(f64.ids()), n + 2, n + 2), dtype=torch.float64, device=dev)
    f32.download_state_device(s32.data_ptr(), len(f32.ids()))
    f64.download_state_device(s64.data_ptr(), len(f64.ids()))
    oa, ob = f32.instance_offsets(), f64.instance_offsets()
    a_all, b_all = f32.ids(), f64.ids()
    rel = np.full(K, np.nan)
    for i in range(K):
        if np.array_equal(a_all[oa[i]:oa[i + 1]], b_all[ob[i]:ob[i + 1]]):
            x = s32[oa[i]:oa[i + 1], h:n + h, h:n + h].double()
            y = s64[ob[i]:ob[i + 1], h:n + h, h:n + h]
            rel[i] = float(torch.linalg.vector_norm(x - y) / torch.linalg.vector_norm(y))
    f32.close()
    f64.close()
    same = parted < 0
    ok = same & np.isfinite(rel)
    return {
        "instances": K, "same_tree_after_every_remesh": int(same.sum()),
        "max_rel_l2_same_history": float(rel[ok].max()) if ok.any() else None,
        "median_rel_l2_same_history": float(np.median(rel[ok])) if ok.any() else None,
        "within_1e-5_same_history": int((rel[ok] <= 1e-5).sum()),
        "parted": int((~same).sum()),
        "first_parting_interval_min": int(parted[~same].min()) if (~same).any() else None,
        "max_rel_l2_parted_same_final_tree": (float(np.nanmax(rel[~same])) if np.isfinite(rel[~same]).any()
                                              else None),
        "note": "an instance parts when a re-mesh of its FP32 run flags differently from its FP64 run (a squared "
                "gradient within rounding of a threshold); from then on the two runs hold different meshes",
    }


def batched_active_extra(args, torch, A, dev, stream, flush, world):
    """The batched forest with level bounds that let it adapt: the trees
    change at the re-meshes, coarse-fine faces appear and the update runs as
    one-step launches.  FP32 throughput, re-mesh counts and leaf range, the
    FP64 run of the same forest, a roofline of the one-step update, and the
    first instances against the oracle."""
    B = BATCHED
    caps, vel, bmp = batched_instances()
    bounds = np.stack([np.maximum(caps - 2, 0), caps], 1).astype(np.int32)
    f32 = make_forest(A, A.F32, stream, caps, vel, bounds)
    ids0 = f32.ids()
    P0 = len(ids0)
    ic64, _ = batched_ic(torch, ids0, bmp, dev)
    ic32 = ic64.to(torch.float32).contiguous()
    # the runs change the forest: each run starts from the refined forest
    snap_ids = ids0.copy()

    def reset(f, ic):
        f.reset()
        f.refine_to_levels(caps)
        assert np.array_equal(f.ids(), snap_ids)
        f.load_state_device(ic.data_ptr(), P0)

    def run(f):
        return f.run(B["steps"], B["remesh"], None, B["cfl"], "grad", B["rthr"], B["cthr"], instance_params=True)

    for _ in range(max(1, args.warmup - 1)):
        reset(f32, ic32)
        run(f32)
    ms, launches, stats, _ = time_runs(torch, stream, world, max(1, args.steps), lambda: reset(f32, ic32),
                                       lambda: run(f32), flush)
    cells = sum(st["cell_updates"] for st in stats)
    st0 = stats[0]
    ids32 = f32.ids()
    s32 = torch.empty((len(ids32), B["n"] + 2, B["n"] + 2), dtype=torch.float32, device=dev)
    f32.download_state_device(s32.data_ptr(), len(ids32))
    # the one-step update timed alone (CUDA events per launch) in a run that
    # continues from the adapted forest, so every launch is a one-step update
    f32.set_timing(True)
    run(f32)
    k_ms, k_launches, k_cells = f32.get_timing()
    f32.set_timing(False)
    # the same forest in FP64
    f64 = make_forest(A, A.F64, stream, caps, vel, bounds)
    reset(f64, ic64)
    ms64, _, stats64, _ = time_runs(torch, stream, world, 1, lambda: reset(f64, ic64), lambda: run(f64), flush)
    ids64 = f64.ids()
    same = bool(np.array_equal(ids64, ids32))
    rel = None
    if same:
        s64 = torch.empty((len(ids64), B["n"] + 2, B["n"] + 2), dtype=torch.float64, device=dev)
        f64.download_state_device(s64.data_ptr(), len(ids64))
        n, h = B["n"], B["halo"]
        a, b = s32[:, h:n + h, h:n + h].double(), s64[:, h:n + h, h:n + h]
        rel = float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
    # FP32 against FP64 per instance, interval by interval: an instance's
    # trees can part where an FP32 gradient and its FP64 counterpart fall on
    # either side of a threshold; after that the states differ by the
    # re-mesh, not by rounding
    hist = precision_history(A, torch, stream, caps, vel, bounds, ic32, ic64, reset, dev)
    # the first instances against the oracle, 100 steps from the same state
    npar, spar = 8, 100
    reset(f64, ic64)
    off = f64.instance_offsets()
    init = [ic64[off[i]:off[i + 1]].cpu().numpy() for i in range(npar)]
    f64.run(spar, B["remesh"], None, B["cfl"], "grad", B["rthr"], B["cthr"], instance_params=True)
    fin = torch.empty((len(f64.ids()), B["n"] + 2, B["n"] + 2), dtype=torch.float64, device=dev)
    f64.download_state_device(fin.data_ptr(), len(f64.ids()))
    o, gids = f64.instance_offsets(), f64.ids()
    mask = np.uint64((1 << (6 + 2 * B["depth"])) - 1)
    _, _, _, finals = cpu_batched(os.cpu_count() or 1, npar, spar, init=init, bounds=bounds)
    trees, worst = True, 0.0
    n, h = B["n"], B["halo"]
    for i, (oids, ost) in enumerate(finals):
        trees &= bool(np.array_equal(gids[o[i]:o[i + 1]] & mask, oids))
        if trees:
            g = fin[o[i]:o[i + 1]].cpu().numpy()[:, h:n + h, h:n + h]
            r = ost[:, h:n + h, h:n + h]
            worst = max(worst, float(np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-300)))
    f32.close()
    f64.close()
    hbm = measured_peaks().get("hbm_gbs")
    achieved = 8.0 * k_cells / (k_ms * 1e-3) / 1e9 if k_ms > 0 else None
    value = cells / (ms * 1e-3)
    return {
        "workload": ACTIVE_NAME,
        "value": value, "unit": UNIT, "ms_per_run": ms / max(1, args.steps), "dtype": "f32",
        "leaves": {"start": P0, "min": int(st0["leaves_min"]), "max": int(st0["leaves_max"]),
                   "mean": float(st0["leaves_mean"])},
        "remeshes": int(st0["remeshes"]), "remeshes_changed": int(st0["remeshes_changed"]),
        "update_share_of_run": (k_ms / (ms / max(1, args.steps))) if ms > 0 else None,
        "gpu_launches": int(launches // max(1, args.steps)),
        "fp64_same_forest": {"value": sum(st["cell_updates"] for st in stats64) / (ms64 * 1e-3), "unit": UNIT,
                             "same_final_tree_as_fp32": same, "rel_l2_fp32_vs_fp64": rel,
                             "per_instance": hist},
        "roofline": {
            "bound": "hbm", "kernel": "k_run_step2d<float,16,1,W,S> (one step per launch: the forest has "
                                      "coarse-fine faces)",
            "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": (achieved / hbm) if achieved and hbm else None,
            "algorithmic_bytes_per_cell_update": 8, "launches": int(k_launches),
            "avg_launch_us": (k_ms * 1e3 / k_launches) if k_launches else None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured, burst copy)" if hbm else "missing",
        },
        "parity": {"sample": f"instances 0-{npar - 1}, {spar} steps, FP64, against the oracle",
                   "trees_bit_exact": trees, "max_instance_rel_l2": worst, "bar": 1e-12,
                   "within_bar": bool(trees and worst <= 1e-12)},
    }


# ----------------------------------------------------- plain FP64 drop-in
def bumps():
    import amr_gb300 as A

    return A.seeded_bumps(2, 2, WORKLOAD["bump_seed"])


def plain_config2(args, torch, A, dev, stream, flush, world):
    """The single-tree active-AMR workload in FP64 through the drop-in."""
    W = WORKLOAD
    tree = A.Tree(W["rank"], W["n"], W["halo"], W["depth"], capacity=4096, stream=stream.cuda_stream)
    tree.refine_uniform(W["init_levels"])
    init = A.gaussian_state(tree.ids(), W["rank"], W["n"], W["halo"], W["depth"], bumps(), W["noise"], W["noise_seed"])
    P0 = init.shape[0]
    init_dev = torch.from_numpy(init).to(f"cuda:{dev}")
    init_host = torch.from_numpy(init).pin_memory()
    final_host = torch.empty((4096,) + init.shape[1:], dtype=torch.float64).pin_memory()
    run_args = dict(steps=W["steps"], interval=W["remesh"], velocity=W["velocity"], cfl=W["cfl"], criterion="grad",
                    rthr=W["rthr"], cthr=W["cthr"], min_level=W["min_level"], max_level=W["max_level"])
    d2h = [0]

    def setup():
        tree.reset()
        tree.refine_uniform(W["init_levels"])

    def body(e2e=False, per_launch=False):
        if e2e:
            A.check(A.lib().amr_tree_upload_state(tree._h, init_host.data_ptr(), P0))
        else:
            tree.load_state_device(init_dev.data_ptr(), P0)
        tree.halo_exchange()
        st = tree.run(per_launch=per_launch, graph=not per_launch, **run_args)
        if e2e:
            P = tree.size
            A.check(A.lib().amr_tree_download_state(tree._h, final_host.data_ptr(), P))
            d2h[0] += P * tree.flat * 8
        return st

    for _ in range(args.warmup):
        setup()
        body()
    ms, launches, stats, _ = time_runs(torch, stream, world, args.steps, setup, body, flush)
    cells = sum(s["cell_updates"] for s in stats)
    for _ in range(args.warmup):  # the host buffers' first transfers are not part of a step
        setup()
        body(e2e=True)
    d2h[0] = 0
    e2e_ms, _, e2e_stats, _ = time_runs(torch, stream, world, args.steps, setup, lambda: body(e2e=True), flush)
    e2e_cells = sum(s["cell_updates"] for s in e2e_stats)
    pl_ms, pl_launches, pl_stats, _ = time_runs(torch, stream, world, 1, setup, lambda: body(per_launch=True), flush)
    pl_cells = sum(s["cell_updates"] for s in pl_stats)
    tree.set_timing(True)
    for _ in range(args.steps):
        setup()
        flush.zero_()
        torch.cuda.synchronize()
        body()
    k_ms, k_launches, k_cells = tree.get_timing()
    tree.set_timing(False)
    tree.close()
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    achieved = 16.0 * k_cells / (k_ms * 1e-3) / 1e9 if k_ms > 0 else None
    traffic = None
    prof = REPO / "profiles" / "k_cycle_fp64_config2.json"
    if prof.exists():
        try:
            traffic = json.loads(prof.read_text()).get("dram_bytes_per_launch")
        except Exception:
            traffic = None
    persistent = all(s["persistent_intervals"] == s["intervals"] for s in stats)
    leaves = [(s["leaves_min"], s["leaves_max"], s["leaves_mean"]) for s in stats]
    return {
        "workload": WORKLOAD_NAME,
        "dtype": "f64",
        "value": cells / (ms * 1e-3),
        "unit": UNIT,
        "ms_per_run": ms / args.steps,
        "leaves_min": int(min(l[0] for l in leaves)),
        "leaves_max": int(max(l[1] for l in leaves)),
        "leaves_mean": float(np.mean([l[2] for l in leaves])),
        "remesh_per_run": int(stats[0]["remeshes"]),
        "sum_dt_per_run": stats[0]["sum_dt"],
        "driver": "one persistent cluster kernel per run" if persistent else "mixed persistent/graph",
        "gpu_launches": int(launches),
        "e2e": {"value": e2e_cells / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(init.nbytes),
                "d2h_bytes_per_step": int(d2h[0] / max(1, args.steps))},
        "roofline": {
            "bound": "hbm", "kernel": "k_cycle<double> (persistent: fused updates, flags, re-mesh)",
            "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": (achieved / hbm) if (achieved and hbm) else None, "traffic": traffic,
            "algorithmic_bytes_per_cell_update": 16,
            "note": "the workload is L2-resident (<= 43 leaves, ~0.1 MB); the figure shows latency, not bandwidth",
        },
        "host_driven": {"value": pl_cells / (pl_ms * 1e-3), "unit": UNIT, "gpu_launches": int(pl_launches),
                        "note": "same runs with host-driven launches and a readback every interval"},
        "cpu_baseline": None,
    }


# ---------------------------------------------- further single-tree workloads
CONFIG3 = dict(rank=3, n=8, halo=1, depth=6, init_levels=1, steps=500, remesh=10, velocity=(1.0, 0.7, 0.3), cfl=0.4,
               rthr=0.05, cthr=0.01, min_level=1, max_level=4, bump_seed=3, bumps=4, sigma=(0.05, 0.08))
# config 2's tree never passes ~43 leaves at max level 5, and the gradient
# criterion at its thresholds stops refining near level 5 whatever the cap;
# the labelled deep variant lowers the thresholds 50x and allows level 8
# (Morton depth 8), which keeps ~4-6k leaves of an adapting tree
DEEP = dict(WORKLOAD, depth=8, init_levels=4, min_level=3, max_level=8, rthr=0.001, cthr=0.0002)
DEEP_NAME = ("2D linear advection, active AMR, FP64 plain, deep variant of config 2: 16x16 patches + 1 ghost, "
             "level 4 start, levels 3-8, grad criterion 0.001/0.0002 (config 2's thresholds / 50), re-mesh every "
             "10 steps, 2 seeded Gaussian bumps, v=(1,0.5), periodic, CFL 0.4, 2000 steps")


def single_tree_runs(torch, A, dev, stream, flush, cfg, dtype, bumps_list, noise, noise_seed, reps):
    """reps timed runs of one configuration from its initial state; returns
    (ms per run, stats of the last run, final interior state, ids)."""
    t = A.Tree(cfg["rank"], cfg["n"], cfg["halo"], cfg["depth"], capacity=1 << 16, dtype=dtype,
               stream=stream.cuda_stream)
    t.refine_uniform(cfg["init_levels"])
    init = A.gaussian_state(t.ids(), cfg["rank"], cfg["n"], cfg["halo"], cfg["depth"], bumps_list, noise, noise_seed)
    P0 = init.shape[0]
    dev_init = torch.from_numpy(init).to(f"cuda:{dev}", torch.float64 if dtype == A.F64 else torch.float32)
    args = dict(steps=cfg["steps"], interval=cfg["remesh"], velocity=cfg["velocity"], cfl=cfg["cfl"],
                criterion="grad", rthr=cfg["rthr"], cthr=cfg["cthr"], min_level=cfg["min_level"],
                max_level=cfg["max_level"])

    def setup():
        t.reset()
        t.refine_uniform(cfg["init_levels"])
        t.load_state_device(dev_init.data_ptr(), P0)

    setup()
    t.run(**args)  # warm-up
    ms, _, stats, _ = time_runs(torch, stream, 1, reps, setup, lambda: t.run(**args), flush)
    out = t.download_state()
    ids = t.ids()
    t.close()
    h, n, r = cfg["halo"], cfg["n"], cfg["rank"]
    inner = out[(slice(None),) + (slice(h, n + h),) * r].astype(np.float64)
    return ms / reps, stats[-1], inner, ids


def config3_extra(torch, A, dev, stream, flush, reps):
    C = CONFIG3
    b = A.seeded_bumps(3, C["bumps"], C["bump_seed"], sigma=C["sigma"])
    ms64, st64, s64, ids64 = single_tree_runs(torch, A, dev, stream, flush, C, A.F64, b, 0.0, 0, reps)
    ms32, st32, s32, ids32 = single_tree_runs(torch, A, dev, stream, flush, C, A.F32, b, 0.0, 0, reps)
    same = np.array_equal(ids64, ids32)
    uniform = {4: {}, 5: {}}
    for lvl, (name, dtype, tdtype, esize) in [(lv, d) for lv in (4, 5) for d in (
            ("fp64", A.F64, torch.float64, 8), ("fp32", A.F32, torch.float32, 4))]:
        # a uniform tree of 8^lvl leaves of 8^3 (level 4: 4096 leaves, 33 MB
        # of FP64 state, L2-resident; level 5: 32768 leaves, 0.26 GB): the
        # staged update kernel's launches timed with CUDA events, 100 steps,
        # no re-mesh
        t = A.Tree(3, C["n"], C["halo"], C["depth"], capacity=8 ** lvl + 64, dtype=dtype, stream=stream.cuda_stream)
        t.refine_uniform(lvl)
        u0 = A.gaussian_state(t.ids(), 3, C["n"], C["halo"], C["depth"], b, 0.0, 0)
        x = torch.from_numpy(u0).to(f"cuda:{dev}", tdtype).contiguous()
        t.load_state_device(x.data_ptr(), t.size)
        t.advance(10, C["velocity"], C["cfl"])
        t.finish_advance()
        t.set_timing(True)
        t.advance(100, C["velocity"], C["cfl"])
        t.finish_advance()
        k_ms, k_n, k_cells = t.get_timing()
        t.set_timing(False)
        t.close()
        hbm = measured_peaks().get("hbm_gbs")
        ach = 2.0 * esize * k_cells / (k_ms * 1e-3) / 1e9 if k_ms > 0 else None
        rec = {"value": k_cells / (k_ms * 1e-3) if k_ms > 0 else None, "launches": k_n,
               "avg_launch_us": k_ms * 1e3 / k_n if k_n else None,
               "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                            "frac": ach / hbm if ach and hbm else None,
                            "algorithmic_bytes_per_cell_update": 2 * esize}}
        if esize == 8:
            # c0 u + sum_a c_a u_a: one DMUL and three DFMA per cell update
            rec["fp64_pipe"] = {"fp64_ops_per_cell_update": 4, "fp64_ops_per_s": 4 * rec["value"] if rec["value"] else
                                None, "note": "the FP64 update is bound by the FP64 pipe (ncu: FP64 pipe 72% active "
                                              "on the level-5 tree), not by HBM"}
        uniform[lvl][name] = rec
    return {
        "uniform_level4": dict(uniform[4], workload="uniform level 4 (4096 leaves of 8^3 + 1 ghost), the staged "
                                                    "update kernel alone (k_step3d), 100 steps, CUDA events per launch"),
        "uniform_level5": dict(uniform[5], workload="uniform level 5 (32768 leaves of 8^3 + 1 ghost), the staged "
                                                    "update kernel alone (k_step3d), 100 steps, CUDA events per launch"),
        "workload": ("3D linear advection with AMR: 8^3 patches + 1 ghost, level 1 start, max level 4, gradient "
                     "criterion 0.05/0.01, re-mesh every 10 steps, 4 seeded Gaussian blobs, v = (1, 0.7, 0.3), "
                     "CFL 0.4, 500 steps"),
        "fp64": {"value": st64["cell_updates"] / (ms64 * 1e-3), "ms_per_run": ms64, "leaves_max": st64["leaves_max"],
                 "leaves_mean": st64["leaves_mean"]},
        "fp32": {"value": st32["cell_updates"] / (ms32 * 1e-3), "ms_per_run": ms32, "leaves_max": st32["leaves_max"]},
        "same_final_tree": bool(same),
        "rel_l2_fp32_vs_fp64": (float(np.linalg.norm(s32 - s64) / np.linalg.norm(s64)) if same else None),
        "unit": UNIT,
    }


def deep_extra(torch, A, dev, stream, flush, reps, with_cpu=True):
    """The deep variant of config 2 (4-6k leaves) in FP64 through the device
    tree: throughput, leaf range, a roofline of the one-step FP64 update on the
    adapted tree, and the oracle on the host cores (timed, and the final tree
    and state compared)."""
    C = DEEP
    t = A.Tree(C["rank"], C["n"], C["halo"], C["depth"], capacity=1 << 15, dtype=A.F64, stream=stream.cuda_stream)
    t.refine_uniform(C["init_levels"])
    init = A.gaussian_state(t.ids(), C["rank"], C["n"], C["halo"], C["depth"], bumps(), C["noise"], C["noise_seed"])
    P0 = init.shape[0]
    dev_init = torch.from_numpy(init).to(f"cuda:{dev}")
    args = dict(steps=C["steps"], interval=C["remesh"], velocity=C["velocity"], cfl=C["cfl"], criterion="grad",
                rthr=C["rthr"], cthr=C["cthr"], min_level=C["min_level"], max_level=C["max_level"])

    def setup():
        t.reset()
        t.refine_uniform(C["init_levels"])
        t.load_state_device(dev_init.data_ptr(), P0)

    setup()
    t.run(**args)  # warm-up
    ms, _, stats, _ = time_runs(torch, stream, 1, reps, setup, lambda: t.run(**args), flush)
    st = stats[-1]
    ids, fin = t.ids(), t.download_state()
    # the one-step update alone, on the adapted tree (a run continuing it)
    t.set_timing(True)
    t.run(**args)
    k_ms, k_launches, k_cells = t.get_timing()
    t.set_timing(False)
    t.close()
    hbm = measured_peaks().get("hbm_gbs")
    achieved = 16.0 * k_cells / (k_ms * 1e-3) / 1e9 if k_ms > 0 else None
    out = {
        "workload": DEEP_NAME, "value": st["cell_updates"] / (ms * 1e-3 / reps), "unit": UNIT, "ms_per_run": ms / reps,
        "dtype": "f64", "leaves_min": st["leaves_min"], "leaves_max": st["leaves_max"],
        "leaves_mean": st["leaves_mean"], "remeshes_changed": st["remeshes_changed"],
        "intervals": {"cluster_kernel": st["persistent_intervals"], "graph": st["graph_intervals"],
                      "total": st["intervals"]},
        "roofline": {"bound": "hbm", "kernel": "k_run_step2d<double,16,1,W,S> (one step per launch)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved and hbm else None, "algorithmic_bytes_per_cell_update": 16,
                     "launches": int(k_launches), "avg_launch_us": (k_ms * 1e3 / k_launches) if k_launches else None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured, burst copy)" if hbm else "missing"},
    }
    if with_cpu:
        from oracle import oracle as O

        threads = os.cpu_count() or 1
        O.set_threads(threads)
        o = O.OracleTree(C["rank"], C["n"], C["halo"], C["depth"], 1 << 15)
        o.refine_all(C["init_levels"])
        o.set_state(init)
        o.halo_exchange()
        t0, done, cells = time.perf_counter(), 0, 0
        while done < C["steps"]:
            leaves = o.size
            _, ex = o.advance(C["remesh"], C["velocity"], C["cfl"])
            done += ex
            cells += ex * leaves * C["n"] ** 2
            f = o.flags_gradient(C["rthr"], C["cthr"], C["min_level"], C["max_level"])
            assert o.reconstruct(f) == 0
            o.halo_exchange()
        secs = time.perf_counter() - t0
        n, h = C["n"], C["halo"]
        same = bool(np.array_equal(ids, o.ids()))
        out["cpu_baseline"] = {"value": cells / secs, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": "the whole run, FP64, OpenMP over patches like EXECUTION=PAR"}
        out["parity"] = {"final_tree_bit_exact": same,
                         "rel_l2": (rel_l2_np(fin[:, h:n + h, h:n + h], o.state()[:, h:n + h, h:n + h])
                                    if same else None), "bar": 1e-12}
    return out


def rel_l2_np(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


# ------------------------------------------------------------- VTK writer
def vtk_extra(torch, A, dev, stream, with_cpu=True):
    """The device-resident VTK writer on the adjoint workload's mesh (2629
    leaves of 16x16, FP64): file size, time of amr_tree_write_vtk (device
    sections + copy-back + file write) and of the oracle's C writer on the same
    tree, and whether the two files are identical."""
    import hashlib
    import tempfile

    J, W = ADJOINT, WORKLOAD
    t, log = adjoint_mesh(A, A.F64, stream)
    u0 = A.gaussian_state(t.ids(), 2, J["n"], J["halo"], J["depth"], bumps(), W["noise"], W["noise_seed"])
    t.upload_state(u0)
    out = {"workload": f"VTK snapshot of the adjoint mesh ({t.size} leaves of 16x16, FP64)"}
    with tempfile.TemporaryDirectory() as d:
        gp = Path(d) / "gpu.vtk"
        t.write_vtk(gp)  # warm-up
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            t.write_vtk(gp)
        gsec = (time.perf_counter() - t0) / reps
        size = gp.stat().st_size
        out.update({"bytes": size, "gpu_seconds": gsec, "gpu_mb_per_s": size / gsec / 1e6})
        if with_cpu:
            from oracle import oracle as O

            O.build()
            o = O.OracleTree(2, J["n"], J["halo"], J["depth"], 40000)
            o.refine_all(J["base_level"])
            for f in log:
                assert o.reconstruct(f) == 0
            o.set_state(u0)
            cp = Path(d) / "cpu.vtk"
            t0 = time.perf_counter()
            o.write_vtk(cp)
            csec = time.perf_counter() - t0
            same = hashlib.sha256(gp.read_bytes()).digest() == hashlib.sha256(cp.read_bytes()).digest()
            out.update({"cpu_seconds": csec, "cpu_mb_per_s": size / csec / 1e6, "cpu_kind": "oracle port, 1 thread",
                        "identical_files": bool(same)})
    t.close()
    return out


# ------------------------------------------------------------ Euler form
# The reference's Euler benchmark (benchmark/bench_fvm_solver_integration.
# b.cpp:34-250): 2D EulerPhysics, 64x64 patches + 1 ghost, Morton depth 7,
# domain 1000 x 1000, three uniform levels, acoustic pulse (rho_bg 0.5, p_bg
# 1, amplitude 10, width^2 = 0.01 L^2, centre (500, 500)), gamma 1.4, CFL
# 0.3, max-Rho criterion 0.53 / 0.49 on levels 1..6, re-mesh every 10
# steps, until t = 50.
EULER = dict(n=64, halo=1, depth=7, lengths=(1000.0, 1000.0), init_levels=3, gamma=1.4, cfl=0.3, end_time=50.0,
             interval=10, rthr=0.53, cthr=0.49, min_level=1, max_level=6, capacity=10000, rho_bg=0.5, p_bg=1.0,
             amp=10.0, width_sq=0.01 * 1000.0 * 1000.0, centre=(500.0, 500.0), cpu_seconds=15.0, cpu_max_intervals=40)


def euler_ic(A, ids):
    """The acoustic pulse at the cell centres, primitive (rho, 0, 0, p) to
    conservative; host array (4, P, n+2, n+2), ghosts zero."""
    E = EULER
    n, h = E["n"], E["halo"]
    x = A.cell_centres(ids, 2, n, E["depth"], E["lengths"])
    r2 = (x[..., 0] - E["centre"][0]) ** 2 + (x[..., 1] - E["centre"][1]) ** 2
    pert = E["amp"] * np.exp(-r2 / E["width_sq"])
    rho = E["rho_bg"] + pert * 0.2
    pres = E["p_bg"] + pert
    st = np.zeros((4, len(ids), n + 2 * h, n + 2 * h))
    st[0][:, h:n + h, h:n + h] = rho
    st[3][:, h:n + h, h:n + h] = pres / (E["gamma"] - 1.0)
    return st


def euler_tree(A, stream, capacity=None):
    E = EULER
    t = A.Tree(2, E["n"], E["halo"], E["depth"], capacity=capacity or E["capacity"], dtype=A.F64,
               lengths=E["lengths"] + (1.0,), stream=stream.cuda_stream, fields=4)
    t.refine_uniform(E["init_levels"])
    st0 = euler_ic(A, t.ids())
    t.upload_state(st0)
    t.halo_exchange()
    return t, st0


def euler_run(t, steps):
    E = EULER
    return t.euler_run(steps, E["interval"], E["gamma"], E["cfl"], E["end_time"], E["rthr"], E["cthr"],
                       E["min_level"], E["max_level"])


def euler_extra(torch, A, stream, with_cpu=True):
    """The reference's Euler benchmark loop to t = 50 through
    amr_tree_euler_run (wall clock around the loop, as the reference times
    it); the step kernels timed with CUDA events on the final mesh; and the
    oracle (C restatement, OpenMP over patches) on the first intervals of the
    same run, whose state the GPU run must reproduce bit for bit."""
    E = EULER
    out = {"workload": "reference Euler benchmark: 2D, 64x64 patches + 1 ghost, acoustic pulse on 1000 x 1000, "
                       "levels 1..6 by max Rho 0.53/0.49, re-mesh every 10 steps, t = 0..50, FP64"}
    t, _ = euler_tree(A, stream)
    euler_run(t, 20)  # warm-up
    t.close()
    t, st0 = euler_tree(A, stream)
    torch.cuda.synchronize()
    l0 = A.launch_count()
    t0 = time.perf_counter()
    st = euler_run(t, 10 ** 9)
    secs = time.perf_counter() - t0
    cells = int(st["cell_updates"])
    flat_cells = cells * (E["n"] + 2 * E["halo"]) ** 2 // E["n"] ** 2
    out.update({"value": cells / secs, "unit": "cell-updates/s (interior cells)", "seconds": secs,
                "reference_count_value": flat_cells / secs,
                "reference_count_note": "the reference's printout counts executed x patches x flat_size (ghosts "
                                        "included, 66^2 per patch)",
                "sim_time": st["sum_dt"], "steps": int(st["executed_steps"]), "remeshes": int(st["remeshes"]),
                "leaves_min": int(st["leaves_min"]), "leaves_max": int(st["leaves_max"]),
                "leaves_final": t.size, "gpu_launches": int(A.launch_count() - l0)})
    # on the final mesh: whole steps (finalize + update + halo) and the
    # update kernel alone (CUDA events on the tree's stream)
    k = 50
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        t.euler_advance(5, E["gamma"], E["cfl"])
        ev0.record(stream)
        t.euler_advance(k, E["gamma"], E["cfl"])
        ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1) / k
    t.set_timing(True)
    t.euler_advance(k, E["gamma"], E["cfl"])
    kms, kl, kcells = t.get_timing()
    t.set_timing(False)
    step_cells = t.size * E["n"] ** 2
    out["final_mesh_step"] = {"ms": ms, "cells": step_cells, "cell_updates_per_s": step_cells / (ms * 1e-3),
                              "update_kernel_ms": kms / kl, "update_kernel_share": (kms / kl) / ms}
    prof = json.loads((REPO / "profiles" / "k_euler_step_fp64_benchmark.json").read_text())
    per_cell = prof["fp64_add_mul_fma_per_cell"]
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    peak = prof["fp64_peak_thread_inst_per_cycle_per_sm"] * sms * measured_peaks().get("sm_max_mhz", 2070.0) * 1e6
    achieved = per_cell * kcells / (kms * 1e-3)
    out["roofline"] = {"bound": "fp64", "achieved": achieved / 1e9, "peak": peak / 1e9, "unit": "G FP64 inst/s",
                       "frac": achieved / peak, "traffic": prof["dram_bytes_per_cell"] * step_cells,
                       "note": f"{per_cell:.0f} FP64 add/mul/fma per cell update (ncu, committed profile) x cells / "
                               f"CUDA-event time of k_euler_step; peak = 2 per cycle per SM x SMs x max SM clock; "
                               f"traffic = DRAM bytes per cell (ncu) x cells of one launch"}
    t.close()
    if with_cpu:
        from oracle import oracle as O

        O.build()
        threads = os.cpu_count() or 1
        O.set_threads(threads)
        o = O.OracleTree(2, E["n"], E["halo"], E["depth"], E["capacity"], nvar=4, lengths=E["lengths"])
        o.refine_all(E["init_levels"])
        o.set_state(np.moveaxis(st0, 0, 1))
        o.halo_exchange()
        ccells, csecs, sim, intervals = 0, 0.0, 0.0, 0
        while csecs < E["cpu_seconds"] and intervals < E["cpu_max_intervals"] and sim < E["end_time"]:
            leaves = o.size
            c0 = time.perf_counter()
            acc, ex, _ = o.euler_advance(E["interval"], E["gamma"], E["cfl"], E["end_time"] - sim)
            f = o.flags_max(E["rthr"], E["cthr"], E["min_level"], E["max_level"])
            assert o.reconstruct(f) == 0
            o.halo_exchange()
            csecs += time.perf_counter() - c0
            sim += acc
            ccells += ex * leaves * E["n"] ** 2
            intervals += 1
        out["cpu_baseline"] = {"value": ccells / csecs, "unit": "cell-updates/s (interior cells)", "cores": threads,
                               "kind": "port", "sample": f"first {intervals} intervals ({intervals * E['interval']} "
                                                         f"steps) of the same run, OpenMP over patches"}
        # the GPU over the same intervals: the state must be the oracle's
        g, _ = euler_tree(A, stream)
        euler_run(g, intervals * E["interval"])
        same_tree = bool(np.array_equal(g.ids(), o.ids()))
        m = np.ones((E["n"] + 2,) * 2, bool)
        m[0, 0] = m[0, -1] = m[-1, 0] = m[-1, -1] = False
        a = g.download_state()[..., m]
        b = np.moveaxis(o.state(), 1, 0)[..., m] if same_tree else None
        out["parity"] = {"intervals": intervals, "same_tree": same_tree,
                         "bit_exact": bool(same_tree and np.array_equal(a, b)),
                         "max_abs_diff": float(np.max(np.abs(a - b))) if same_tree else None}
        g.close()
    return out


# ------------------------------------------------------------ SSPRK form
# SSPRK2 / SSPRK3 steps (the reference's integrators on the FV advection
# residual) on a uniform level-7 tree of 16x16 patches (16384 patches, 4.2 M
# cells), FP64, velocity (1, 0.5), CFL 0.4, Gaussian bumps plus noise.
SSPRK = dict(n=16, halo=1, depth=8, level=7, steps=60, cfl=0.4, velocity=(1.0, 0.5), cpu_steps=4)


def ssprk_extra(torch, A, stream, with_cpu=True):
    """SSPRK steps through amr_tree_advance_ssprk (CUDA events on the tree's
    stream around `steps` steps), and the oracle on the host cores for a few
    steps of the same tree; the states must agree bit for bit."""
    S, W = SSPRK, WORKLOAD
    out = {"workload": f"SSPRK2/3 advection, uniform level {S['level']} of 16x16 patches + 1 ghost (FP64), "
                       f"{S['steps']} steps, CFL {S['cfl']}, v = {S['velocity']}"}
    for order in (2, 3):
        t = A.Tree(2, S["n"], S["halo"], S["depth"], capacity=20000, dtype=A.F64, stream=stream.cuda_stream)
        t.refine_uniform(S["level"])
        u0 = A.gaussian_state(t.ids(), 2, S["n"], S["halo"], S["depth"], bumps(), W["noise"], W["noise_seed"])
        t.upload_state(u0)
        t.halo_exchange()
        t.advance_ssprk(4, order, S["velocity"], S["cfl"])  # warm-up
        t.finish_advance()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            ev0.record(stream)
            t.advance_ssprk(S["steps"], order, S["velocity"], S["cfl"])
            ev1.record(stream)
        ev1.synchronize()
        _, ex = t.finish_advance()
        ms = ev0.elapsed_time(ev1)
        cells = ex * t.size * S["n"] ** 2
        rate = cells / (ms * 1e-3)
        alg = 3 * 8 * order  # per stage: read the stage input and u^n, write the result (FP64)
        hbm = measured_peaks().get("hbm_gbs")
        rec = {"value": rate, "unit": "cell-updates/s", "ms_per_step": ms / ex, "leaves": t.size,
               "roofline": {"bound": "hbm", "achieved": alg * rate / 1e9, "peak": hbm, "unit": "GB/s",
                            "frac": alg * rate / 1e9 / hbm if hbm else None,
                            "algorithmic_bytes_per_cell_update": alg,
                            "note": "each stage reads its input and u^n and writes its output once (halo "
                                    "exchanges and neighbour reads beside)"}}
        if with_cpu:
            from oracle import oracle as O

            O.build()
            threads = os.cpu_count() or 1
            O.set_threads(threads)
            o = O.OracleTree(2, S["n"], S["halo"], S["depth"], 40000)
            o.refine_all(S["level"])
            o.set_state(u0)
            o.halo_exchange()
            c0 = time.perf_counter()
            _, cex = o.ssprk_advance(S["cpu_steps"], order, S["velocity"], S["cfl"])
            csec = time.perf_counter() - c0
            g = A.Tree(2, S["n"], S["halo"], S["depth"], capacity=20000, dtype=A.F64, stream=stream.cuda_stream)
            g.refine_uniform(S["level"])
            g.upload_state(u0)
            g.halo_exchange()
            g.advance_ssprk(S["cpu_steps"], order, S["velocity"], S["cfl"])
            g.finish_advance()
            rec["cpu_baseline"] = {"value": cex * o.size * S["n"] ** 2 / csec, "unit": "cell-updates/s",
                                   "cores": threads, "kind": "port",
                                   "sample": f"first {S['cpu_steps']} steps of the same tree, OpenMP over patches"}
            rec["parity_first_steps_bit_exact"] = bool(np.array_equal(g.download_state(), o.state()))
            g.close()
        t.close()
        out[f"ssprk{order}"] = rec
    return out


# ------------------------------------------------------------ DG patch solver
# The reference's DG configuration (order 2, 2D, 4x4 cells per patch, four
# advected variables per node, SSPRK2, velocity 1): its own main loop runs a
# uniform level-5 start (1024 leaves); the throughput line uses level 9
# (262144 leaves, 4.2 M cells, 16 nodal values each: 1.2 GB per state buffer).
DG = dict(levels=(5, 9), steps={5: 200, 9: 20}, dt0=0.01, cpu_level=5, cpu_steps=3)


def dg_extra(torch, A, stream, with_cpu=True):
    """DG steps through amr_tree_dg_advance (CUDA events on the tree's stream
    around the timed steps, after the first step at the initial dt), and the
    numpy restatement on the host for a few steps of the level-5 tree; the
    states must agree bit for bit."""
    from oracle import dg_oracle as G

    D = DG
    out = {"workload": "nodal DG advection (the reference's dg_helpers configuration: order 2, 2D, 4x4 cells per "
                       "patch + 1 ghost, 4 variables per node, SSPRK2, velocity 1, initial dt 0.01 then the CFL "
                       "step), uniform levels, no re-mesh",
           "unit": "cell-updates/s (interior cells, each with 16 nodal values)"}
    for lv in D["levels"]:
        t = A.Tree(2, 4, 1, 10, capacity=(1 << (2 * lv)) + 64, dtype=A.F64, fields=16, stream=stream.cuda_stream)
        t.refine_uniform(lv)
        cells = t.size * 16
        # the initial nodal field of the reference's scenario, built per patch
        # on the host from the restatement (sin at the nodes)
        u0 = np.zeros((16, t.size, 6, 6))
        U = G.initial_state(lv) if lv <= 6 else None
        if U is not None:
            u0 = _dg_fields(G.to_leaves(U, lv))
        else:
            rng = np.random.default_rng(11)
            u0[:, :, 1:5, 1:5] = rng.uniform(-1.0, 1.0, (16, t.size, 4, 4))
        t.upload_state(u0)
        dt, tm = t.dg_advance(1, D["dt0"])  # the first step at the initial dt; warm-up
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n = D["steps"][lv]
        with torch.cuda.stream(stream):
            ev0.record(stream)
            dt, tm = t.dg_advance(n, dt, tm)
            ev1.record(stream)
        ev1.synchronize()
        ms = ev0.elapsed_time(ev1)
        rate = cells * n / (ms * 1e-3)
        # per stage the kernel reads the stage input (16 x 8 B per cell; the
        # neighbours' values come from L1/L2) and, in the second stage, u^n,
        # and writes the result: 2 + 3 = 5 x 128 B per cell and step
        alg = 5 * 128
        hbm = measured_peaks().get("hbm_gbs")
        rec = {"value": rate, "unit": "cell-updates/s", "ms_per_step": ms / n, "leaves": t.size, "cells": cells,
               "steps_timed": n, "dt_after": dt,
               "roofline": {"bound": "hbm", "achieved": alg * rate / 1e9, "peak": hbm, "unit": "GB/s",
                            "frac": alg * rate / 1e9 / hbm if hbm else None,
                            "algorithmic_bytes_per_cell_update": alg,
                            "note": "two stages per step, each reads its input state and writes its output; "
                                    "the second also reads u^n; the FP64 arithmetic (about 1100 operations "
                                    "per cell and step, no contraction) is the likelier bound"}}
        if with_cpu and lv == D["cpu_level"]:
            L0 = D["cpu_level"]
            U0 = G.initial_state(L0)
            c0 = time.perf_counter()
            outs, _ = G.run(L0, D["cpu_steps"], dt0=D["dt0"], U=U0)
            csec = time.perf_counter() - c0
            g = A.Tree(2, 4, 1, 10, capacity=(1 << (2 * L0)) + 64, dtype=A.F64, fields=16,
                       stream=stream.cuda_stream)
            g.refine_uniform(L0)
            g.upload_state(_dg_fields(G.to_leaves(U0, L0)))
            g.dg_advance(D["cpu_steps"], D["dt0"])
            mine = _dg_leaves(g.download_state())
            rec["cpu_baseline"] = {"value": (16 << (2 * L0)) * D["cpu_steps"] / csec, "unit": "cell-updates/s",
                                   "cores": 1, "kind": "port",
                                   "sample": f"first {D['cpu_steps']} steps of the level-{L0} tree, numpy "
                                             "restatement (vectorised over cells, one thread)"}
            rec["parity_first_steps_bit_exact"] = bool(np.array_equal(mine, G.to_leaves(outs[-1], L0)))
            g.close()
        t.close()
        out[f"level{lv}"] = rec
    out["solver_loop"] = dg_loop(torch, A, stream)
    return out


def dg_loop(torch, A, stream):
    """The reference's DG main loop (examples/dg_main_loop.e.cpp with
    DGSolver::run, solver.hpp:109-151): uniform level 5, initial dt 0.01,
    re-mesh every 20 steps with thresholds 0.05 / 0.01, until t = 1; the
    reference's count of processed cells (leaves x 16 per step) over the wall
    time of the loop (host-driven: one call per step and per re-mesh)."""
    from oracle import dg_oracle as G

    L0 = 5
    u0 = _dg_fields(G.to_leaves(G.initial_state(L0), L0))
    best = None
    for _ in range(2):  # the first run includes the first use of the kernels
        t = A.Tree(2, 4, 1, 6, capacity=8192, dtype=A.F64, fields=16, stream=stream.cuda_stream)
        t.refine_uniform(L0)
        t.upload_state(u0)
        torch.cuda.synchronize()
        c0 = time.perf_counter()
        st = t.dg_run(0.01, 1.0, 20, 0.05, 0.01)
        sec = time.perf_counter() - c0
        t.close()
        if best is None or sec < best[0]:
            best = (sec, st)
    sec, st = best
    return {"value": st["cells"] / sec, "unit": "cell-updates/s (the reference's processed cells/s)", "seconds": sec,
            "steps": st["steps"], "remeshes": st["remeshes"], "leaves_max": st["leaves_max"], "sim_time": st["time"],
            "driver": "amr_tree_dg_run: the loop in one call (host-driven launches, a leaf-count readback per "
                      "re-mesh)"}


DG_EULER = dict(levels=(5, 9), steps={5: 100, 9: 10}, dt0={5: 0.003, 9: 1e-5}, cpu_level=5, cpu_steps=3)


def _dg_euler_pulse(lv):
    """The reference's DG Euler initial state (pressure pulse exp(-100 r^2) + 1
    at the nodes, rho 1, zero momentum), vectorised for large levels: the
    tree's [field, leaf, 6, 6] in the Morton leaf order of a uniform level."""
    P, C = 4, 4 << lv
    cell = (1.0 / float(1 << lv)) / 4.0
    pts = (0.5 - 0.5 / np.sqrt(3.0), 0.5 + 0.5 / np.sqrt(3.0))
    c = (np.arange(C) + 0.5) * cell
    n = 1 << lv
    m = np.arange(n * n, dtype=np.int64)
    px = np.zeros_like(m)
    py = np.zeros_like(m)
    for bit in range(lv):
        px |= ((m >> (2 * bit)) & 1) << bit
        py |= ((m >> (2 * bit + 1)) & 1) << bit
    a = np.zeros((16, n * n, 6, 6))
    for ix in range(2):
        for iy in range(2):
            x = c[None, :] + (pts[ix] - 0.5) * cell
            y = c[:, None] + (pts[iy] - 0.5) * cell
            p = np.exp(-100.0 * ((x - 0.5) ** 2 + (y - 0.5) ** 2)) + 1.0  # [cy, cx]
            blk = p.reshape(n, P, n, P).transpose(0, 2, 1, 3)[py, px]     # [leaf, ly, lx]
            k = ix * 2 + iy
            a[k * 4 + 2, :, 1:5, 1:5] = 1.0
            a[k * 4 + 3, :, 1:5, 1:5] = blk / (1.4 - 1.0)
    return a


def dg_euler_extra(torch, A, stream, with_cpu=True):
    """DG Euler steps (the reference's DG Euler equations in the same order-2
    configuration: pressure pulse, CFL step from the patches' wave speeds)
    through amr_tree_dg_advance; the numpy restatement on the host for a few
    steps of the level-5 tree, bit for bit."""
    from oracle import dg_oracle as G

    D = DG_EULER
    out = {"workload": "nodal DG Euler (order 2, 2D, 4x4 cells per patch + 1 ghost, variables [rho u, rho v, rho, "
                       "E] per node, SSPRK2, Rusanov speed = the patch's running maximum, CFL step from the last "
                       "stage), pressure pulse, uniform levels, no re-mesh",
           "unit": "cell-updates/s (interior cells, each with 16 nodal values)"}
    for lv in D["levels"]:
        t = A.Tree(2, 4, 1, 10, capacity=(1 << (2 * lv)) + 64, dtype=A.F64, fields=16, stream=stream.cuda_stream)
        t.dg_set_equation("euler")
        t.refine_uniform(lv)
        cells = t.size * 16
        t.upload_state(_dg_euler_pulse(lv))
        dt, tm = t.dg_advance(1, D["dt0"][lv])  # warm-up: the first step at the initial dt
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n = D["steps"][lv]
        with torch.cuda.stream(stream):
            ev0.record(stream)
            dt, tm = t.dg_advance(n, dt, tm)
            ev1.record(stream)
        ev1.synchronize()
        ms = ev0.elapsed_time(ev1)
        rate = cells * n / (ms * 1e-3)
        rec = {"value": rate, "unit": "cell-updates/s", "ms_per_step": ms / n, "leaves": t.size, "cells": cells,
               "steps_timed": n, "dt_after": dt,
               "launches_per_step": 7,
               "note": "per step: two halo exchanges, two primitive passes (p, u, v per node), two stages and "
                       "the step-size update; the step size stays on the device"}
        if with_cpu and lv == D["cpu_level"]:
            L0 = D["cpu_level"]
            U0 = G.euler_initial_state(L0)
            c0 = time.perf_counter()
            outs, _ = G.run(L0, D["cpu_steps"], dt0=D["dt0"][L0], U=U0, equation="euler")
            csec = time.perf_counter() - c0
            g = A.Tree(2, 4, 1, 10, capacity=(1 << (2 * L0)) + 64, dtype=A.F64, fields=16,
                       stream=stream.cuda_stream)
            g.dg_set_equation("euler")
            g.refine_uniform(L0)
            g.upload_state(_dg_fields(G.to_leaves(U0, L0)))
            g.dg_advance(D["cpu_steps"], D["dt0"][L0])
            mine = _dg_leaves(g.download_state())
            rec["cpu_baseline"] = {"value": (16 << (2 * L0)) * D["cpu_steps"] / csec, "unit": "cell-updates/s",
                                   "cores": 1, "kind": "port",
                                   "sample": f"first {D['cpu_steps']} steps of the level-{L0} tree, numpy "
                                             "restatement (vectorised over cells, the running maximum in a "
                                             "Python loop, one thread)"}
            rec["parity_first_steps_bit_exact"] = bool(np.array_equal(mine, G.to_leaves(outs[-1], L0)))
            g.close()
        t.close()
        out[f"level{lv}"] = rec
    return out


def _dg_fields(st):
    """[leaf, cell, node, var] -> the tree's [field, leaf, 6, 6] (ghosts zero)."""
    P = st.shape[0]
    a = np.zeros((16, P, 6, 6))
    a[:, :, 1:5, 1:5] = st.reshape(P, 4, 4, 4, 4).transpose(3, 4, 0, 1, 2).reshape(16, P, 4, 4)
    return a


def _dg_leaves(a):
    P = a.shape[1]
    return a[:, :, 1:5, 1:5].reshape(4, 4, P, 4, 4).transpose(2, 3, 4, 0, 1).reshape(P, 16, 4, 4)


# ------------------------------------------------------------ adjoint form
ADJOINT = dict(n=16, halo=1, depth=8, base_level=5, max_level=7, rthr=0.01, cthr=0.002, rounds=3, steps=400,
               every=20, cfl=0.4, velocity=(1.0, 0.5), directions=64, eps=1e-4, pert=0.05, seed=7)


def adjoint_mesh(A, dtype, stream, flag_log=None):
    """Frozen mesh: config 2's initial field (two seeded bumps + noise) on a
    uniform level-5 base, adapted at step 0 by the gradient criterion (0.01 /
    0.002, up to level 7), three rounds.  flag_log replays recorded flags."""
    J, W = ADJOINT, WORKLOAD
    t = A.Tree(2, J["n"], J["halo"], J["depth"], capacity=40000, dtype=dtype, stream=stream.cuda_stream)
    t.refine_uniform(J["base_level"])
    log = []
    for r in range(J["rounds"]):
        if flag_log is None:
            t.upload_state(A.gaussian_state(t.ids(), 2, J["n"], J["halo"], J["depth"], bumps(), W["noise"],
                                            W["noise_seed"]))
            t.flags_gradient(J["rthr"], J["cthr"], J["base_level"], J["max_level"])
            f = t.get_flags()
        else:
            f = flag_log[r]
            t.set_flags(f)
        log.append(f)
        t.remesh()
    return t, log


def adjoint_extra(torch, A, dev, stream, with_oracle=True):
    J, W = ADJOINT, WORKLOAD
    t64, log = adjoint_mesh(A, A.F64, stream)
    t32, _ = adjoint_mesh(A, A.F32, stream, log)
    ids = t64.ids()
    assert np.array_equal(ids, t32.ids())
    P = len(ids)
    n, h = J["n"], J["halo"]
    u0_np = A.gaussian_state(ids, 2, n, h, J["depth"], bumps(), W["noise"], W["noise_seed"])
    mask = torch.zeros(u0_np.shape, dtype=torch.bool, device=f"cuda:{dev}")
    mask[:, h:n + h, h:n + h] = True
    u0 = torch.from_numpy(u0_np).to(f"cuda:{dev}")
    rng = np.random.default_rng(J["seed"])
    pert = torch.from_numpy(rng.standard_normal(u0_np.shape)).to(f"cuda:{dev}") * mask

    def run(tree, u, dtype):
        x = u.to(dtype).contiguous()
        tree.load_state_device(x.data_ptr(), P)
        tree.advance(J["steps"], J["velocity"], J["cfl"])
        tree.finish_advance()
        out = torch.empty_like(x)
        tree.download_state_device(out.data_ptr(), P)
        return out

    target = run(t64, u0 + J["pert"] * pert, torch.float64)

    def loss64(u):
        r = (run(t64, u, torch.float64) - target) * mask
        return 0.5 * torch.sum(r * r)

    res = {}
    for name, tree, dt in (("f64", t64, torch.float64), ("f32", t32, torch.float32)):
        adj = A.Adjoint(tree, J["steps"], J["velocity"], J["cfl"], every=J["every"])
        x = u0.to(dt).contiguous()
        lam0 = torch.empty_like(x)
        fw, bw = [], []
        for rep in range(4):
            tree.load_state_device(x.data_ptr(), P)
            torch.cuda.synchronize()
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            adj.forward()
            e1.record(stream)
            uT = torch.empty_like(x)
            tree.download_state_device(uT.data_ptr(), P)
            r = ((uT - target.to(dt)) * mask).contiguous()
            torch.cuda.synchronize()
            e1b = torch.cuda.Event(enable_timing=True)
            e1b.record(stream)
            adj.backward(r.data_ptr(), lam0.data_ptr())
            e2.record(stream)
            torch.cuda.synchronize()
            if rep:  # first repetition warms up
                fw.append(e0.elapsed_time(e1))
                bw.append(e1b.elapsed_time(e2))
        res[name] = dict(uT=uT.double(), grad=lam0.double(), r=r.double(), fw_ms=float(np.median(fw)),
                         bw_ms=float(np.median(bw)))
        adj.close()
    g = res["f64"]["grad"]
    # central finite differences of the FP64 loss along seeded directions
    worst, errs = 0.0, []
    for _ in range(J["directions"]):
        v = torch.from_numpy(rng.standard_normal(u0_np.shape)).to(f"cuda:{dev}") * mask
        fd = (loss64(u0 + J["eps"] * v) - loss64(u0 - J["eps"] * v)) / (2 * J["eps"])
        gv = torch.sum(g * v)
        e = float(abs(fd - gv) / abs(gv))
        errs.append(e)
        worst = max(worst, e)

    def rel(a, b):
        return float(torch.linalg.vector_norm((a - b)[mask]) / torch.linalg.vector_norm(b[mask]))

    out = {
        "workload": (f"adjoint: frozen 2D mesh of {P} leaves (16x16 + 1 ghost; config-2 initial field on a uniform "
                     f"level-{J['base_level']} base adapted at step 0 up to level {J['max_level']}), velocity "
                     f"{J['velocity']}, CFL {J['cfl']}, {J['steps']} steps, checkpoint every {J['every']}; loss "
                     f"0.5||u_T - u_target||^2, u_target = the solver's image of u_0 + {J['pert']} x seeded noise"),
        "leaves": P,
        "cost_ratio_fp64": res["f64"]["bw_ms"] / res["f64"]["fw_ms"],
        "cost_ratio_fp32": res["f32"]["bw_ms"] / res["f32"]["fw_ms"],
        "forward_ms": {"f64": res["f64"]["fw_ms"], "f32": res["f32"]["fw_ms"]},
        "backward_ms": {"f64": res["f64"]["bw_ms"], "f32": res["f32"]["bw_ms"]},
        "fd_check": {"directions": J["directions"], "eps": J["eps"], "max_rel_err": worst,
                     "median_rel_err": float(np.median(errs)), "bar": 1e-6, "within_bar": bool(worst <= 1e-6),
                     "precision": "FP64 forward and adjoint"},
        "fp32": {"rel_l2_uT_vs_fp64": rel(res["f32"]["uT"], res["f64"]["uT"]),
                 "rel_l2_grad_vs_fp64": rel(res["f32"]["grad"], g)},
        "cost_bar": 3.0,
    }
    if with_oracle:
        from oracle import oracle as O

        O.build()
        O.set_threads(os.cpu_count() or 1)
        o = O.OracleTree(2, n, h, J["depth"], 40000)
        o.refine_all(J["base_level"])
        for f in log:
            assert o.reconstruct(f) == 0
        assert np.array_equal(o.ids(), ids)
        o.set_state(u0_np)
        o.halo_exchange()
        t0 = time.perf_counter()
        ref = o.adjoint(J["steps"], J["velocity"], J["cfl"], res["f64"]["r"].cpu().numpy())
        secs = time.perf_counter() - t0
        ref_t = torch.from_numpy(ref).to(f"cuda:{dev}")
        out["oracle_reference_gradient"] = {"rel_l2_gpu_fp64": rel(g, ref_t), "rel_l2_gpu_fp32": rel(res["f32"]["grad"], ref_t),
                                            "cpu_seconds": secs, "threads": os.cpu_count() or 1}
    t64.close()
    t32.close()
    return out


def uniform_extra(A, torch, stream, dtype, level=9, steps=40):
    """Kernel-level figure on an HBM-sized input: uniform 2D tree of 4^level
    leaves (16x16 + 1 ghost), fused update only (no re-mesh), per-launch
    kernels timed with CUDA events on the tree's stream.  Each step streams
    both state buffers (> L2), so no flush is needed."""
    elem = 8 if dtype == A.F64 else 4
    t = A.Tree(2, 16, 1, level, capacity=4**level, dtype=dtype, stream=stream.cuda_stream)
    t.refine_uniform(level)
    rng = np.random.default_rng(5)
    t.upload_state(rng.random((t.size, 18, 18)))
    t.advance(5, (1.0, 0.5), 0.4)
    t.finish_advance()
    t.set_timing(True)
    torch.cuda.synchronize()
    e0, e1 = _events(torch)
    e0.record(stream)
    t.advance(steps, (1.0, 0.5), 0.4)
    e1.record(stream)
    acc, ex = t.finish_advance()
    ms = e0.elapsed_time(e1)
    k_ms, k_launches, k_cells = t.get_timing()
    t.close()
    hbm = measured_peaks().get("hbm_gbs")
    achieved = elem * 2 * k_cells / (k_ms * 1e-3) / 1e9
    out = {
        "workload": f"uniform 2D tree, 4^{level} = {4**level} leaves of 16x16 + 1 ghost, {steps} steps, no re-mesh",
        "dtype": "f64" if dtype == A.F64 else "f32",
        "value": ex * 4**level * 256 / (ms * 1e-3),
        "unit": UNIT,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm if hbm else None, "algorithmic_bytes_per_cell_update": 2 * elem,
                     "avg_launch_us": k_ms * 1e3 / max(1, k_launches)},
    }
    if dtype == A.F64:
        # the FP64 pipe is the ceiling here: 1 DMUL + 2 DFMA per 2D cell update
        dfma = 3 * k_cells / (k_ms * 1e-3)
        out["fp64_pipe"] = {"achieved_ops_per_s": dfma, "peak_ops_per_s": 0.60e12,
                            "frac": dfma / 0.60e12, "peak_source": "FMA-throughput probe on this GB300 pool"}
    return out


def aggregate_replicas(torch, device, ms, e2e_ms, cells, e2e_cells):
    """Whole-job figures of N independent replicas: the slowest rank's time
    (max) and the sum of the cell updates of all ranks."""
    t = torch.tensor([ms, e2e_ms], dtype=torch.float64, device=device)
    c = torch.tensor([float(cells), float(e2e_cells)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.all_reduce(c, op=torch.distributed.ReduceOp.SUM)
    ms, e2e_ms = t.tolist()
    cells, e2e_cells = c.tolist()
    return ms, e2e_ms, cells, e2e_cells


def gpu_arm(args, rank, world):
    import torch

    import amr_gb300 as A

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{dev}")
    bt = batched_arm(args, torch, A, dev, stream, flush, world)
    extras = {}
    if not args.no_extras:
        cpu = not args.no_cpu_baseline
        table = {
            "batched_active": lambda: batched_active_extra(args, torch, A, dev, stream, flush, world),
            "plain_fp64_config2": lambda: plain_config2(args, torch, A, dev, stream, flush, world),
            "adjoint": lambda: adjoint_extra(torch, A, dev, stream, with_oracle=cpu),
            "config3_3d": lambda: config3_extra(torch, A, dev, stream, flush, max(1, args.steps)),
            "vtk_writer": lambda: vtk_extra(torch, A, dev, stream, with_cpu=cpu),
            "plain_fp64_config2_deep": lambda: deep_extra(torch, A, dev, stream, flush, max(1, args.steps), with_cpu=cpu),
            "euler_benchmark": lambda: euler_extra(torch, A, stream, with_cpu=cpu),
            "ssprk_advection": lambda: ssprk_extra(torch, A, stream, with_cpu=cpu),
            "dg_advection": lambda: dg_extra(torch, A, stream, with_cpu=cpu),
            "dg_euler": lambda: dg_euler_extra(torch, A, stream, with_cpu=cpu),
        }
        for name, fn in table.items():
            if args.extra is None or name in args.extra:
                extras[name] = fn()
        if args.uniform:
            lv = args.uniform_level
            extras[f"uniform_fp64_level{lv}"] = uniform_extra(A, torch, stream, A.F64, lv)
            extras[f"uniform_fp32_level{lv}"] = uniform_extra(A, torch, stream, A.F32, lv)
    ms, e2e_ms, cells, e2e_cells = bt["ms"], bt["e2e_ms"], bt["cells"], bt["e2e_cells"]
    if world > 1:
        ms, e2e_ms, cells, e2e_cells = aggregate_replicas(torch, f"cuda:{dev}", ms, e2e_ms, cells, e2e_cells)
    if rank != 0:
        return None
    bt["e2e"]["value"] = e2e_cells / (e2e_ms * 1e-3)
    cfg = dict(bt["config"])
    cfg["parallelism"] = f"replicas x{world}" if world > 1 else "single GPU"
    line = {
        "metric": METRIC,
        "value": cells / (ms * 1e-3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded per-instance caps, velocities and Gaussian bumps; shapes of the named config)",
        "config": cfg,
        "e2e": bt["e2e"],
        "roofline": bt["roofline"],
        "fp64_plain_same_workload": bt["fp64_plain_same_workload"],
        "precision": bt["precision"],
        "clocks": bt["clocks"],
        "gpu_launches": int(bt["launches"]),
        "_parity": bt["parity"],
    }
    line.update(extras)
    return line


# ------------------------------------------------------------------ CPU arms
def cpu_batched(threads: int, instances: int, steps: int, init=None, bounds=None):
    """The oracle (C restatement of the reference) on the host cores: the
    first `instances` instances of the batched workload, each a separate
    tree, truncated to `steps` steps.  init: per instance the padded FP64
    initial state the GPU forest starts from (else the oracle's own bumps);
    bounds: per-instance (min, max) levels (default: held at the cap).
    Returns the cell updates, the seconds of the loops, the caps, and per
    instance the final (Morton ids, padded state)."""
    from oracle import oracle as O

    O.set_threads(threads)
    B = BATCHED
    caps, vel, bmp = batched_instances()
    cells, secs, finals = 0, 0.0, []
    for i in range(instances):
        lo, hi = (int(caps[i]), int(caps[i])) if bounds is None else (int(bounds[i][0]), int(bounds[i][1]))
        t = O.OracleTree(2, B["n"], B["halo"], B["depth"], int(4 ** hi) * 2 + 64)
        t.refine_all(int(caps[i]))
        if init is None:
            t.init_state([float(v) for v in bmp[i].ravel()])
        else:
            t.set_state(init[i])
        t.halo_exchange()
        t0 = time.perf_counter()
        done = 0
        while done < steps:
            k = min(B["remesh"], steps - done)
            leaves = t.size
            _, ex = t.advance(k, tuple(vel[i]), B["cfl"])
            done += ex
            cells += ex * leaves * B["n"] ** 2
            f = t.flags_gradient(B["rthr"], B["cthr"], lo, hi)
            if t.reconstruct(f) != 0:
                raise RuntimeError("oracle re-mesh failed")
            t.halo_exchange()
            if ex == 0:
                break
        secs += time.perf_counter() - t0
        finals.append((t.ids(), t.state()))
    return cells, secs, caps[:instances], finals


CPU_SAMPLE = dict(instances=32, steps=100)


def parity_report(par, finals):
    """The headline forest against the oracle on the CPU baseline's sample:
    per instance the final leaves (bit-exact) and the relative L2 of the
    interior state, GPU FP64 (bar 1e-12) and GPU FP32 (bar 1e-5)."""
    n, h = BATCHED["n"], BATCHED["halo"]
    out = {"sample": f"instances 0-{len(finals) - 1}, {par['steps']} steps from the GPU forest's initial state, "
                     f"against the oracle (FP64, C restatement pinned to the reference)"}
    for key, bar in (("f64", 1e-12), ("f32", 1e-5)):
        trees, worst = True, 0.0
        for (gids, gst), (oids, ost) in zip(par[key], finals):
            trees &= bool(np.array_equal(np.asarray(gids, np.uint64), np.asarray(oids, np.uint64)))
            a, b = gst[:, h:n + h, h:n + h], ost[:, h:n + h, h:n + h]
            worst = max(worst, float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)))
        out[key] = {"trees_bit_exact": trees, "max_instance_rel_l2": worst, "bar": bar,
                    "within_bar": bool(trees and worst <= bar)}
    return out


def cpu_baseline(init=None):
    """The timed CPU sample; with init (the GPU forest's initial states of the
    sampled instances) also the sample's final trees and states."""
    threads = os.cpu_count() or 1
    cells, secs, caps, finals = cpu_batched(threads, CPU_SAMPLE["instances"], CPU_SAMPLE["steps"], init=init)
    return {"value": cells / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"instances 0-{CPU_SAMPLE['instances'] - 1} of the batched workload ({int(np.sum(4 ** caps))} "
                      f"patches), first {CPU_SAMPLE['steps']} steps each from the GPU forest's initial state, FP64, "
                      f"OpenMP over patches like EXECUTION=PAR"}, finals


def cpu_plain(steps=600):
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    W = WORKLOAD
    t0 = time.perf_counter()
    _, _, _, cells, _ = O.run_scenario(
        W["rank"], W["n"], W["halo"], W["depth"], init_levels=W["init_levels"], steps=steps, remesh=W["remesh"],
        velocity=W["velocity"], cfl=W["cfl"], bumps=bumps(), noise=W["noise"], noise_seed=W["noise_seed"],
        crit="grad", rthr=W["rthr"], cthr=W["cthr"], min_level=W["min_level"], max_level=W["max_level"],
        capacity=4096)
    secs = time.perf_counter() - t0
    return {"value": cells / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {steps} of the 2000 steps, OpenMP over patches like EXECUTION=PAR"}


def reference_arm(args, rank, world):
    if rank != 0:
        return None
    from oracle import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    cpu_batched(threads, 4, 20)  # warm-up: page in, thread pool
    for _ in range(max(0, args.warmup - 1)):
        cpu_batched(threads, 4, 20)
    total_cells, total_s, caps = 0, 0.0, None
    for _ in range(args.steps):
        c, s, caps, _ = cpu_batched(threads, CPU_SAMPLE["instances"], CPU_SAMPLE["steps"])
        total_cells += c
        total_s += s
    value = total_cells / total_s
    sample = (f"instances 0-{CPU_SAMPLE['instances'] - 1} of the batched workload ({int(np.sum(4 ** caps))} patches), "
              f"first {CPU_SAMPLE['steps']} steps each, FP64; the C restatement of the reference, pinned bit-exact to "
              f"the reference's own runs (its sources are not on this host, so the reference itself cannot be built "
              f"here), OpenMP over patches")
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_s * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded per-instance caps, velocities and Gaussian bumps; shapes of the named config)",
        "config": {"workload": BATCHED_NAME, "sample": f"instances 0-{CPU_SAMPLE['instances'] - 1}, first "
                                                      f"{CPU_SAMPLE['steps']} steps each",
                   "comparison": "rate of a bounded FP64 sample of the same workload on the host cores against "
                                 "the GPU arm's rate over the whole forest in FP32: a rate ratio across "
                                 "precisions, as the metric (FP32 batched against FP64) asks"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def profile_case(name, steps):
    """One untimed run of a workload, for profilers: forest (the batched FP32
    forest, `steps` steps), adjoint (the adjoint mesh, FP64 forward and
    backward over `steps` steps), config2 (one config-2 run), euler (the Euler
    benchmark's first `steps` steps), dg_euler (`steps` DG Euler steps of the
    uniform level-8 pressure pulse: 65536 leaves, 0.6 GB of state)."""
    import torch

    import amr_gb300 as A

    stream = torch.cuda.Stream()
    if name in ("forest", "forest64", "active"):
        B = BATCHED
        caps, vel, bmp = batched_instances()
        bounds = np.stack([np.maximum(caps - 2, 0), caps], 1).astype(np.int32) if name == "active" else None
        f = make_forest(A, A.F64 if name == "forest64" else A.F32, stream, caps, vel, bounds)
        ids = f.ids()
        ic64, _ = batched_ic(torch, ids, bmp, 0)
        ic = ic64 if name == "forest64" else ic64.to(torch.float32).contiguous()
        f.load_state_device(ic.data_ptr(), len(ids))
        st = f.run(steps, B["remesh"], None, B["cfl"], "grad", B["rthr"], B["cthr"], instance_params=True)
    elif name == "deep":
        C = DEEP
        t = A.Tree(C["rank"], C["n"], C["halo"], C["depth"], capacity=1 << 15, stream=stream.cuda_stream)
        t.refine_uniform(C["init_levels"])
        t.upload_state(A.gaussian_state(t.ids(), C["rank"], C["n"], C["halo"], C["depth"], bumps(), C["noise"],
                                        C["noise_seed"]))
        st = t.run(steps=steps, interval=C["remesh"], velocity=C["velocity"], cfl=C["cfl"], criterion="grad",
                   rthr=C["rthr"], cthr=C["cthr"], min_level=C["min_level"], max_level=C["max_level"])
    elif name == "adjoint":
        J = ADJOINT
        t, _ = adjoint_mesh(A, A.F64, stream)
        u0 = A.gaussian_state(t.ids(), 2, J["n"], J["halo"], J["depth"], bumps(), WORKLOAD["noise"],
                              WORKLOAD["noise_seed"])
        x = torch.from_numpy(u0).cuda().contiguous()
        t.load_state_device(x.data_ptr(), t.size)
        adj = A.Adjoint(t, steps, J["velocity"], J["cfl"], every=J["every"])
        adj.forward()
        lam, out = torch.ones_like(x), torch.empty_like(x)
        adj.backward(lam.data_ptr(), out.data_ptr())
        st = {"leaves": t.size, "steps": steps}
    elif name in ("uniform3d", "uniform3d32"):
        # a uniform level-5 3D tree (32768 leaves of 8^3 + 1 ghost, 0.26 GB of
        # FP64 state per buffer, above L2): `steps` update steps, no re-mesh
        C = CONFIG3
        dtype = A.F32 if name == "uniform3d32" else A.F64
        t = A.Tree(3, C["n"], C["halo"], C["depth"], capacity=32768 + 64, dtype=dtype, stream=stream.cuda_stream)
        t.refine_uniform(5)
        b = A.seeded_bumps(3, C["bumps"], C["bump_seed"], sigma=C["sigma"])
        t.upload_state(A.gaussian_state(t.ids(), 3, C["n"], C["halo"], C["depth"], b, 0.0, 0))
        t.advance(steps, C["velocity"], C["cfl"])
        t.finish_advance()
        st = {"leaves": t.size, "steps": steps}
    elif name in ("config3", "config3_32"):
        # one full 3D config-3 run (500 steps, re-mesh every 10)
        C = CONFIG3
        dtype = A.F32 if name == "config3_32" else A.F64
        t = A.Tree(3, C["n"], C["halo"], C["depth"], capacity=1 << 16, dtype=dtype, stream=stream.cuda_stream)
        t.refine_uniform(C["init_levels"])
        b = A.seeded_bumps(3, C["bumps"], C["bump_seed"], sigma=C["sigma"])
        t.upload_state(A.gaussian_state(t.ids(), 3, C["n"], C["halo"], C["depth"], b, 0.0, 0))
        st = t.run(steps=C["steps"], interval=C["remesh"], velocity=C["velocity"], cfl=C["cfl"], criterion="grad",
                   rthr=C["rthr"], cthr=C["cthr"], min_level=C["min_level"], max_level=C["max_level"])
    elif name in ("ssprk2", "ssprk3"):
        # `steps` SSPRK steps of the SSPRK workload (uniform level 7 of 16x16, FP64)
        S, W = SSPRK, WORKLOAD
        t = A.Tree(2, S["n"], S["halo"], S["depth"], capacity=20000, dtype=A.F64, stream=stream.cuda_stream)
        t.refine_uniform(S["level"])
        t.upload_state(A.gaussian_state(t.ids(), 2, S["n"], S["halo"], S["depth"], bumps(), W["noise"],
                                        W["noise_seed"]))
        t.halo_exchange()
        t.advance_ssprk(steps, 2 if name == "ssprk2" else 3, S["velocity"], S["cfl"])
        _, ex = t.finish_advance()
        st = {"leaves": t.size, "steps": ex}
    elif name == "euler":
        t, _ = euler_tree(A, stream, capacity=4000)  # about 1.5 GB of state and primitives
        st = euler_run(t, steps)
    elif name == "dg_euler":
        lv = 8
        t = A.Tree(2, 4, 1, 10, capacity=(1 << (2 * lv)) + 64, dtype=A.F64, fields=16, stream=stream.cuda_stream)
        t.dg_set_equation("euler")
        t.refine_uniform(lv)
        t.upload_state(_dg_euler_pulse(lv))
        dt, tm = t.dg_advance(1, 2e-5)  # first use: scratch allocation
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            ev0.record(stream)
            dt, tm = t.dg_advance(steps, dt, tm)
            ev1.record(stream)
        ev1.synchronize()
        ms = ev0.elapsed_time(ev1) / max(1, steps)
        st = {"leaves": t.size, "steps": steps, "dt": dt, "time": tm, "ms_per_step": ms,
              "cell_updates_per_s": t.size * 16 / (ms * 1e-3)}
    else:
        W = WORKLOAD
        t = A.Tree(2, W["n"], W["halo"], W["depth"], capacity=4096, stream=stream.cuda_stream)
        t.refine_uniform(W["init_levels"])
        t.upload_state(A.gaussian_state(t.ids(), 2, W["n"], W["halo"], W["depth"], bumps(), W["noise"],
                                        W["noise_seed"]))
        t.halo_exchange()
        st = t.run(steps=W["steps"], interval=W["remesh"], velocity=W["velocity"], cfl=W["cfl"], criterion="grad",
                   rthr=W["rthr"], cthr=W["cthr"], min_level=W["min_level"], max_level=W["max_level"])
    torch.cuda.synchronize()
    print(json.dumps({"case": name, "stats": {k: (v if isinstance(v, (int, float)) else str(v))
                                              for k, v in dict(st).items()}}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--uniform", action="store_true", help="add the uniform kernel-level workloads")
    ap.add_argument("--uniform-level", type=int, default=9)
    ap.add_argument("--extra", action="append", default=None,
                    help="run only the named extra workloads after the headline (repeatable)")
    ap.add_argument("--case", choices=["forest", "forest64", "active", "deep", "adjoint", "config2", "euler",
                                       "dg_euler", "uniform3d", "uniform3d32", "config3", "config3_32", "ssprk2",
                                       "ssprk3"],
                    help="run one workload once, untimed (for profilers), and exit")
    ap.add_argument("--case-steps", type=int, default=30)
    args = ap.parse_args()
    if args.case:
        profile_case(args.case, args.case_steps)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        line = reference_arm(args, rank, world)
        if line:
            print(json.dumps(line), flush=True)
        return
    if world > 1:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    line = gpu_arm(args, rank, world)
    if line is not None:
        par = line.pop("_parity", None)
        if not args.no_cpu_baseline:
            line["cpu_baseline"], finals = cpu_baseline(init=par["init"] if par else None)
            if par:
                line["parity"] = parity_report(par, finals)
            if "plain_fp64_config2" in line:
                line["plain_fp64_config2"]["cpu_baseline"] = cpu_plain()
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
