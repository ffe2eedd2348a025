#!/usr/bin/env python
"""Benchmark of the GB300 AMR hot path: cell-updates/s.

Workload (one bench step = one complete run of it): 2D linear advection with
active AMR, plain FP64: 16x16-cell patches + 1 ghost layer, Morton depth 7 with
refinement capped at level 5 by the criterion, gradient criterion
max|grad u|*h > 0.05 refine / < 0.01 coarsen (min level 1), re-mesh every 10
steps with 2:1 balance, two seeded Gaussian bumps (sigma 0.02-0.06, amplitude
0.5-2) plus 1e-3 seeded noise, velocity (1.0, 0.5), periodic, CFL 0.4, 2000
steps.  cell-updates = sum over re-mesh intervals of executed steps x leaves
x 16^2, re-mesh time included (the reference's definition,
benchmark/bench_fvm_solver_integration_active_amr.b.cpp:244-245, 258).

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


def bumps():
    import amr_gb300 as A

    return A.seeded_bumps(2, 2, WORKLOAD["bump_seed"])


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
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    achieved = elem * 2 * k_cells / (k_ms * 1e-3) / 1e9
    out = {
        "workload": f"uniform 2D tree, 4^{level} = {4**level} leaves of 16x16 + 1 ghost, {steps} steps, no re-mesh",
        "dtype": "f64" if dtype == A.F64 else "f32",
        "value": ex * 4**level * 256 / (ms * 1e-3),
        "unit": UNIT,
        "roofline": {"bound": "hbm", "kernel": f"k_step<{'double' if dtype == A.F64 else 'float'}>",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm if hbm else None,
                     "algorithmic_bytes_per_cell_update": 2 * elem,
                     "avg_launch_us": k_ms * 1e3 / max(1, k_launches)},
    }
    if dtype == A.F64:
        # the FP64 pipe is the ceiling here: 1 DMUL + 2 DFMA per 2D cell update
        dfma = 3 * k_cells / (k_ms * 1e-3)
        out["fp64_pipe"] = {"achieved_ops_per_s": dfma, "peak_ops_per_s": 0.60e12,
                            "frac": dfma / 0.60e12, "peak_source": "FMA-throughput probe on this GB300 pool"}
    return out


def gpu_arm(args, rank, world):
    import torch

    import amr_gb300 as A

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()
    W = WORKLOAD
    tree = A.Tree(W["rank"], W["n"], W["halo"], W["depth"], capacity=4096, stream=stream.cuda_stream)
    tree.refine_uniform(W["init_levels"])
    init = A.gaussian_state(tree.ids(), W["rank"], W["n"], W["halo"], W["depth"], bumps(), W["noise"], W["noise_seed"])
    P0 = init.shape[0]
    init_dev = torch.from_numpy(init).to(f"cuda:{dev}")
    init_host = torch.from_numpy(init).pin_memory()
    final_host = torch.empty((4096,) + init.shape[1:], dtype=torch.float64).pin_memory()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{dev}")
    run_args = dict(steps=W["steps"], interval=W["remesh"], velocity=W["velocity"], cfl=W["cfl"], criterion="grad",
                    rthr=W["rthr"], cthr=W["cthr"], min_level=W["min_level"], max_level=W["max_level"])

    def setup():
        # topology of the initial tree: outside the timed interval, as in the
        # reference benchmark (its timer starts after initialisation)
        tree.reset()
        tree.refine_uniform(W["init_levels"])

    def run(e2e: bool, per_launch=False):
        if e2e:
            A.check(A.lib().amr_tree_upload_state(tree._h, init_host.data_ptr(), P0))
        else:
            tree.load_state_device(init_dev.data_ptr(), P0)
        tree.halo_exchange()
        st = tree.run(per_launch=per_launch, **run_args)
        d2h = 0
        if e2e:
            P = tree.size
            A.check(A.lib().amr_tree_download_state(tree._h, final_host.data_ptr(), P))
            d2h = P * tree.flat * 8
        return st, d2h

    def timed(e2e: bool, k: int, per_launch=False):
        total_ms, launches, d2h_total, stats = 0.0, 0, 0, []
        for _ in range(k):
            setup()
            flush.zero_()
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            l0 = A.launch_count()
            ev0, ev1 = _events(torch)
            ev0.record(stream)
            st, d2h = run(e2e, per_launch)
            ev1.record(stream)
            torch.cuda.synchronize()
            launches += A.launch_count() - l0
            total_ms += ev0.elapsed_time(ev1)
            d2h_total += d2h
            stats.append(st)
        return total_ms, launches, d2h_total, stats

    for _ in range(args.warmup):
        setup()
        run(False)
    clocks = ClockSampler(dev)
    clocks.start()
    ms, launches, _, stats = timed(False, args.steps)
    clock_info = clocks.stop()
    cells = sum(s["cell_updates"] for s in stats)
    e2e_ms, _, d2h_total, e2e_stats = timed(True, args.steps)
    e2e_cells = sum(s["cell_updates"] for s in e2e_stats)
    pl_ms, pl_launches, _, pl_stats = timed(False, 1, per_launch=True)
    pl_cells = sum(s["cell_updates"] for s in pl_stats)

    # dominant kernel over a second pass of the same timed runs, CUDA events
    # around every launch of it on the tree's stream
    tree.set_timing(True)
    for _ in range(args.steps):
        setup()
        flush.zero_()
        torch.cuda.synchronize()
        run(False)
    k_ms, k_launches, k_cells = tree.get_timing()
    tree.set_timing(False)

    extras = {}
    if not args.no_extras:
        lv = args.uniform_level
        extras[f"uniform_fp64_level{lv}"] = uniform_extra(A, torch, stream, A.F64, lv)
        extras[f"uniform_fp32_level{lv}"] = uniform_extra(A, torch, stream, A.F32, lv)

    if world > 1:
        t = torch.tensor([ms, e2e_ms], dtype=torch.float64, device=f"cuda:{dev}")
        c = torch.tensor([float(cells), float(e2e_cells)], dtype=torch.float64, device=f"cuda:{dev}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(c, op=torch.distributed.ReduceOp.SUM)
        ms, e2e_ms = t.tolist()
        cells, e2e_cells = c.tolist()
    if rank != 0:
        return None
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    alg_bytes = 16.0 * k_cells  # one read + one write of an FP64 cell per update
    achieved = alg_bytes / (k_ms * 1e-3) / 1e9 if k_ms > 0 else None
    traffic = None
    prof = REPO / "profiles" / "k_cycle_fp64_config2.json"
    if prof.exists():
        try:
            traffic = json.loads(prof.read_text()).get("dram_bytes_per_launch")
        except Exception:
            traffic = None
    persistent = all(s["persistent_intervals"] == s["intervals"] for s in stats)
    leaves = [(s["leaves_min"], s["leaves_max"], s["leaves_mean"]) for s in stats]
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
        "dtype": "f64",
        "data": "synthetic (seeded Gaussian bumps + seeded noise, shapes of the named config)",
        "config": {
            "workload": WORKLOAD_NAME,
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "l2": "flushed (256 MiB write) before every timed run, outside the timed interval",
            "step": "one complete 2000-step run (200 re-meshes) from the initial state",
            "leaves_min": int(min(l[0] for l in leaves)),
            "leaves_max": int(max(l[1] for l in leaves)),
            "leaves_mean": float(np.mean([l[2] for l in leaves])),
            "remesh_per_run": int(stats[0]["remeshes"]),
            "sum_dt_per_run": stats[0]["sum_dt"],
            "driver": "one persistent cluster kernel per run" if persistent else "mixed persistent/per-launch",
        },
        "e2e": {
            "value": e2e_cells / (e2e_ms * 1e-3),
            "unit": UNIT,
            "h2d_bytes_per_step": int(init.nbytes),
            "d2h_bytes_per_step": int(d2h_total / max(1, args.steps)),
        },
        "roofline": {
            "bound": "hbm",
            "kernel": "k_cycle<double> (persistent: fused updates, flags, re-mesh)" if persistent else "k_step<double>",
            "achieved": achieved,
            "peak": hbm,
            "unit": "GB/s",
            "frac": (achieved / hbm) if (achieved and hbm) else None,
            "traffic": traffic,
            "algorithmic_bytes_per_cell_update": 16,
            "launches": k_launches,
            "avg_launch_us": (k_ms * 1e3 / k_launches) if k_launches else None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if hbm else "missing",
            "note": "the workload is L2-resident (<= 43 leaves, ~0.1 MB); the figure shows latency, not bandwidth",
        },
        "per_launch_driver": {"value": pl_cells / (pl_ms * 1e-3), "unit": UNIT, "gpu_launches": int(pl_launches),
                              "note": "same runs with per-launch kernels and host round trips each interval"},
        "clocks": clock_info,
        "gpu_launches": int(launches),
    }
    line.update(extras)
    return line


# ------------------------------------------------------------------ CPU arms
def cpu_run(threads: int, steps: int):
    """The oracle (C restatement of the reference) on the host cores: the same
    workload, truncated to `steps` time steps."""
    from oracle import oracle as O

    O.set_threads(threads)
    W = WORKLOAD
    t0 = time.perf_counter()
    _, sum_dt, done, cells, _ = O.run_scenario(
        W["rank"], W["n"], W["halo"], W["depth"], init_levels=W["init_levels"], steps=steps, remesh=W["remesh"],
        velocity=W["velocity"], cfl=W["cfl"], bumps=bumps(), noise=W["noise"], noise_seed=W["noise_seed"],
        crit="grad", rthr=W["rthr"], cthr=W["cthr"], min_level=W["min_level"], max_level=W["max_level"],
        capacity=4096)
    return cells, time.perf_counter() - t0


def cpu_baseline(steps=600):
    threads = os.cpu_count() or 1
    cells, secs = cpu_run(threads, steps)
    return {"value": cells / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {steps} of the 2000 steps ({steps // WORKLOAD['remesh']} re-meshes), "
                      f"OpenMP over patches like EXECUTION=PAR"}


def reference_arm(args, rank, world):
    if rank != 0:
        return None
    from oracle import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    steps = WORKLOAD["steps"]
    for _ in range(args.warmup):
        cpu_run(threads, 200)
    total_cells, total_s = 0, 0.0
    for _ in range(args.steps):
        c, s = cpu_run(threads, steps)
        total_cells += c
        total_s += s
    value = total_cells / total_s
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
        "data": "synthetic (seeded Gaussian bumps + seeded noise, shapes of the named config)",
        "config": {"workload": WORKLOAD_NAME},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "full 2000-step run per step; the C restatement of the reference "
                                   "(the reference's own build is x86-only here), OpenMP over patches"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--extras-only", action="store_true", help="only the uniform kernel-level workloads")
    ap.add_argument("--uniform-level", type=int, default=9)
    args = ap.parse_args()
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
    if args.extras_only:
        import torch

        import amr_gb300 as A

        stream = torch.cuda.Stream()
        out = {f"uniform_fp64_level{args.uniform_level}": uniform_extra(A, torch, stream, A.F64, args.uniform_level),
               f"uniform_fp32_level{args.uniform_level}": uniform_extra(A, torch, stream, A.F32, args.uniform_level)}
        print(json.dumps(out), flush=True)
        return
    line = gpu_arm(args, rank, world)
    if line is not None:
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline()
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
