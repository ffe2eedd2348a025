"""Generate the golden fixtures in this folder from the REAL reference.

Builds oracle/_ref/ref_driver (the unmodified gpu-amr headers compiled by
oracle/Makefile; needs the reference checkout, so this runs only where it is
present) and records each scenario below as a compressed .npz:

  ids[k]     sorted Morton ids after re-mesh k       (bit-exact pins)
  kind/nbid/quad[k]  neighbour tables in linear-index form
  flags[k]   refine/coarsen status fed to re-mesh k
  state_*    cell states (interior, or full padded for the tree cases)

Usage:  python tests/golden/make_golden.py [--ref /path/to/reference]
"""
from __future__ import annotations

import argparse
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(HERE))
from dumps import TAG_DT, TAG_FLAGS, TAG_STATE, TAG_TREE, read_records  # noqa: E402

DRIVER = REPO / "oracle" / "_ref" / "ref_driver"


def seeded_bumps(rank, count, seed, sigma=(0.02, 0.06), amp=(0.5, 2.0), lo=0.15, hi=0.85):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        c = rng.uniform(lo, hi, size=rank)
        out.extend(list(c) + [rng.uniform(*sigma), rng.uniform(*amp)])
    return [float(round(x, 6)) for x in out]


def linear_neighbors(ids, nb):
    """Neighbour table with Morton ids replaced by linear indices."""
    pos = {int(k): i for i, k in enumerate(ids)}
    kind = nb["kind"].astype(np.int8)
    nbid = np.full(nb["ids"].shape, -1, np.int32)
    P, D, _ = nbid.shape
    n_finer = 2 ** (D // 2 - 1)
    for p in range(P):
        for d in range(D):
            k = kind[p, d]
            if k in (1, 3):
                nbid[p, d, 0] = pos[int(nb["ids"][p, d, 0])]
            elif k == 2:
                for f in range(n_finer):
                    nbid[p, d, f] = pos[int(nb["ids"][p, d, f])]
    quad = nb["quadrant"].astype(np.int8)
    quad[kind != 3] = 0
    return kind, nbid, quad


def run(args, path):
    cmd = [str(DRIVER)] + [f"{k}={v}" for k, v in args.items()] + [f"out={path}"]
    res = subprocess.run(cmd, check=True, capture_output=True, text=True)
    return json.loads(res.stdout.strip().splitlines()[-1])


def scenario_run(name, cfg, rank, n, h, params, state_every=None):
    tmp = Path("/tmp") / f"golden_{name}.bin"
    args = dict(cfg=cfg, mode="run", **params)
    if state_every:
        args["state_every"] = state_every
    info = run(args, tmp)
    recs = read_records(str(tmp), rank)
    trees = [r for r in recs if r[0] == TAG_TREE]
    flags = [r for r in recs if r[0] == TAG_FLAGS]
    states = [r for r in recs if r[0] == TAG_STATE]
    dt = [r for r in recs if r[0] == TAG_DT][0][2]
    P1 = n + 2 * h
    sl = (slice(None),) + (slice(h, n + h),) * rank
    out = {
        "meta": np.array(json.dumps({"cfg": cfg, "rank": rank, "n": n, "halo": h, "depth": 7,
                                     "params": params, "info": info})),
        "sum_dt": np.float64(dt[0]),
        "steps": np.int64(dt[1]),
        "init_ids": trees[0][2]["ids"],
        "state_init": states[0][2].reshape((-1,) + (P1,) * rank)[sl],
        "state_final": states[-1][2].reshape((-1,) + (P1,) * rank)[sl],
        "final_ids": (trees[-1][2]["ids"] if len(trees) > 1 else trees[0][2]["ids"]),
        "n_remesh": np.int64(len(flags)),
    }
    for k, (fl, tr) in enumerate(zip(flags, trees[1:])):
        ids = tr[2]["ids"]
        kind, nbid, quad = linear_neighbors(ids, tr[2]["nb"])
        out[f"step_{k}"] = np.int64(fl[1])
        out[f"flags_{k}"] = fl[2]
        out[f"ids_{k}"] = ids
        out[f"kind_{k}"] = kind
        out[f"nbid_{k}"] = nbid
        out[f"quad_{k}"] = quad
    mids = states[1:-1]
    for j, s in enumerate(mids):
        out[f"state_mid_{j}"] = s[2].reshape((-1,) + (P1,) * rank)[sl]
        out[f"state_mid_step_{j}"] = np.int64(s[1])
    np.savez_compressed(HERE / f"{name}.npz", **out)
    return info


def scenario_tree(name, cfg, rank, n, h, params, keep_states=None):
    tmp = Path("/tmp") / f"golden_{name}.bin"
    info = run(dict(cfg=cfg, mode="tree", **params), tmp)
    recs = read_records(str(tmp), rank)
    trees = [r for r in recs if r[0] == TAG_TREE]
    flags = [r for r in recs if r[0] == TAG_FLAGS]
    states = [r for r in recs if r[0] == TAG_STATE]
    P1 = n + 2 * h
    out = {
        "meta": np.array(json.dumps({"cfg": cfg, "rank": rank, "n": n, "halo": h, "depth": 7,
                                     "params": params, "info": info})),
        "passes": np.int64(len(flags)),
        "ids_init": trees[0][2]["ids"],
        "state_init": states[0][2].reshape((-1,) + (P1,) * rank),
    }
    for k, (fl, tr, st) in enumerate(zip(flags, trees[1:], states[1:])):
        ids = tr[2]["ids"]
        kind, nbid, quad = linear_neighbors(ids, tr[2]["nb"])
        out[f"flags_{k}"] = fl[2]
        out[f"ids_{k}"] = ids
        out[f"kind_{k}"] = kind
        out[f"nbid_{k}"] = nbid
        out[f"quad_{k}"] = quad
        if keep_states is None or k in keep_states:
            out[f"state_{k}"] = st[2].reshape((-1,) + (P1,) * rank)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    return info


def scenario_euler(name, cfg, rank, n, h, params):
    """The reference's amr_solver with EulerPhysics<rank> on the acoustic
    pulse (domain 1000^rank): trees and flags after every re-mesh, initial
    and final states (all fields), simulated time."""
    nvar = rank + 2
    tmp = Path("/tmp") / f"golden_{name}.bin"
    info = run(dict(cfg=cfg, mode="euler", **params), tmp)
    recs = read_records(str(tmp), rank)
    trees = [r for r in recs if r[0] == TAG_TREE]
    flags = [r for r in recs if r[0] == TAG_FLAGS]
    states = [r for r in recs if r[0] == TAG_STATE]
    (time, steps) = [r for r in recs if r[0] == TAG_DT][0][2]
    P1 = n + 2 * h
    out = {
        "meta": np.array(json.dumps({"cfg": cfg, "rank": rank, "n": n, "halo": h, "depth": 7, "nvar": nvar,
                                     "lengths": [1000.0] * rank, "params": params, "info": info})),
        "remeshes": np.int64(len(flags)),
        "ids_init": trees[0][2]["ids"],
        "state_init": states[0][2].reshape((-1, nvar) + (P1,) * rank),
        "state_final": states[-1][2].reshape((-1, nvar) + (P1,) * rank),
        "time": np.float64(time),
        "steps": np.int64(steps),
    }
    for k, (fl, tr) in enumerate(zip(flags, trees[1:])):
        ids = tr[2]["ids"]
        kind, nbid, quad = linear_neighbors(ids, tr[2]["nb"])
        out[f"flags_{k}"] = fl[2]
        out[f"ids_{k}"] = ids
        out[f"kind_{k}"] = kind
        out[f"nbid_{k}"] = nbid
        out[f"quad_{k}"] = quad
    np.savez_compressed(HERE / f"{name}.npz", **out)
    return info


EULER_SCENARIOS = [
    # the reference Euler benchmark's set-up on smaller patches: 8x8 + 1 ghost,
    # 3 uniform levels, max-Rho criterion 0.53 / 0.49 on levels 1..4, gamma 1.4,
    # CFL 0.3, re-mesh every 10 steps
    ("euler_pulse_2d", "2d8h1", 2, 8, 1, dict(init_levels=3, steps=60, remesh=10, max_level=4, min_level=1,
                                              gamma=1.4, cfl=0.3)),
    ("euler_pulse_3d", "3d4h1", 3, 4, 1, dict(init_levels=2, steps=30, remesh=10, max_level=3, min_level=1,
                                              gamma=1.4, cfl=0.3)),
]


def scenario_ssprk(name, cfg, rank, n, h, params):
    """The reference's SSPRK2 / SSPRK3 classes driving the FV advection
    residual patch by patch (halo exchange before every stage), CFL step,
    gradient re-mesh: trees and flags after every re-mesh, initial and final
    padded states, simulated time."""
    tmp = Path("/tmp") / f"golden_{name}.bin"
    info = run(dict(cfg=cfg, mode="ssprk", **params), tmp)
    recs = read_records(str(tmp), rank)
    trees = [r for r in recs if r[0] == TAG_TREE]
    flags = [r for r in recs if r[0] == TAG_FLAGS]
    states = [r for r in recs if r[0] == TAG_STATE]
    (time, steps) = [r for r in recs if r[0] == TAG_DT][0][2]
    P1 = n + 2 * h
    out = {
        "meta": np.array(json.dumps({"cfg": cfg, "rank": rank, "n": n, "halo": h, "depth": 7,
                                     "params": params, "info": info})),
        "remeshes": np.int64(len(flags)),
        "ids_init": trees[0][2]["ids"],
        "state_init": states[0][2].reshape((-1,) + (P1,) * rank),
        "state_final": states[-1][2].reshape((-1,) + (P1,) * rank),
        "time": np.float64(time),
        "steps": np.int64(steps),
    }
    for k, (fl, tr) in enumerate(zip(flags, trees[1:])):
        out[f"flags_{k}"] = fl[2]
        out[f"ids_{k}"] = tr[2]["ids"]
    np.savez_compressed(HERE / f"{name}.npz", **out)
    return info


SSPRK_SCENARIOS = [
    # 2D advection, 8x8 patches + 1 ghost, two uniform levels, two seeded
    # bumps plus noise, gradient re-mesh every 10 steps (levels 1..4), CFL 0.4
    ("ssprk2_advection_2d", "2d8h1", 2, 8, 1, dict(order=2, init_levels=2, steps=30, remesh=10, vel="1,0.5", cfl=0.4,
                                                    bumps="0.3,0.3,0.05,1,0.7,0.6,0.04,1.5", noise=1e-3, noise_seed=3,
                                                    rthr=0.05, cthr=0.01, min_level=1, max_level=4)),
    ("ssprk3_advection_2d", "2d8h1", 2, 8, 1, dict(order=3, init_levels=2, steps=30, remesh=10, vel="-0.7,0.4",
                                                    cfl=0.4, bumps="0.35,0.6,0.05,1,0.65,0.3,0.04,1.5", noise=1e-3,
                                                    noise_seed=4, rthr=0.05, cthr=0.01, min_level=1, max_level=4)),
    ("ssprk3_advection_3d", "3d4h1", 3, 4, 1, dict(order=3, init_levels=2, steps=12, remesh=6, vel="0.6,-0.5,0.8",
                                                    cfl=0.4, bumps="0.4,0.5,0.6,0.08,1.2", noise=1e-3, noise_seed=5,
                                                    rthr=0.05, cthr=0.01, min_level=1, max_level=3)),
]


VTK_SCENARIOS = {
    # name of the npz fixture whose final tree and state are printed -> driver arguments
    "config1_uniform_2d": ("2d8h1", dict(mode="run", init_levels=2, steps=100, remesh=0, vel="1,0.5", cfl=0.4,
                                         bumps="0.3,0.3,0.05,1", noise=1e-3, noise_seed=1, crit="none")),
    "tree_random_2d_n8": ("2d8h1", dict(mode="tree", seed=12, passes=6, init_levels=1, max_level=5, min_level=1,
                                        p_refine=0.3, p_coarsen=0.4)),
    "tree_random_3d_n4": ("3d4h1", dict(mode="tree", seed=13, passes=5, init_levels=1, max_level=4, min_level=1,
                                        p_refine=0.25, p_coarsen=0.5)),
    "tree_random_2d_h2": ("2d10h2", dict(mode="tree", seed=14, passes=4, init_levels=1, max_level=4, min_level=1,
                                         p_refine=0.3, p_coarsen=0.5)),
}


def vtk_golden():
    """The reference's VTK writer (include/ndtree/vtk_print.hpp) on the final
    tree and state of four fixtures: SHA-256 and length of each file."""
    import hashlib
    import tempfile

    out = {}
    for name, (cfg, params) in VTK_SCENARIOS.items():
        with tempfile.TemporaryDirectory() as d:
            cmd = ([str(DRIVER), f"cfg={cfg}"] + [f"{k}={v}" for k, v in params.items()]
                   + [f"out={d}/dump.bin", f"vtk={name}"])
            subprocess.run(cmd, check=True, capture_output=True, text=True, cwd=d)
            data = (Path(d) / "vtk_output" / f"{name}.vtk").read_bytes()
        out[name] = {"sha256": hashlib.sha256(data).hexdigest(), "bytes": len(data), "field": "Scalar"}
    # the Euler pulse fixtures: every field, domain lengths 1000
    for name, cfg, rank, _, _, params in EULER_SCENARIOS:
        with tempfile.TemporaryDirectory() as d:
            cmd = ([str(DRIVER), f"cfg={cfg}", "mode=euler"] + [f"{k}={v}" for k, v in params.items()]
                   + [f"out={d}/dump.bin", f"vtk={name}"])
            subprocess.run(cmd, check=True, capture_output=True, text=True, cwd=d)
            data = (Path(d) / "vtk_output" / f"{name}.vtk").read_bytes()
        names = ["Rho", "Rhou", "Rhov"] + (["Rhow"] if rank == 3 else []) + [f"E{rank}D"]
        out[name] = {"sha256": hashlib.sha256(data).hexdigest(), "bytes": len(data), "field": ",".join(names)}
    (HERE / "vtk.json").write_text(json.dumps(out, indent=1) + "\n")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None,
                    help="reference checkout (default: $AMR_REFERENCE, else the location oracle/Makefile names)")
    ap.add_argument("--vtk-only", action="store_true", help="only the VTK writer fixture")
    ap.add_argument("--euler-only", action="store_true", help="only the Euler fixtures")
    ap.add_argument("--ssprk-only", action="store_true", help="only the SSPRK fixtures")
    a = ap.parse_args()
    ref = a.ref or subprocess.run(["make", "-s", "-C", str(REPO / "oracle"), "print-ref"], check=True,
                                  capture_output=True, text=True).stdout.strip()
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle"), "ref", f"REF={ref}"], check=True)
    if a.vtk_only:
        print(vtk_golden())
        return
    if a.euler_only:
        for sc in EULER_SCENARIOS:
            print(scenario_euler(*sc))
        return
    if a.ssprk_only:
        for sc in SSPRK_SCENARIOS:
            print(scenario_ssprk(*sc))
        return

    # 1: 2D uniform depth 2, 16 leaves of 8x8, FP64, 100 steps, config as in the
    #    reference's config.yaml: CFL 0.4, v = (1, 0.5), Gaussian at (0.3,0.3)
    #    sigma 0.05 amplitude 1, plus seeded uniform noise 1e-3.
    print(scenario_run("config1_uniform_2d", "2d8h1", 2, 8, 1, dict(
        init_levels=2, steps=100, remesh=0, vel="1,0.5", cfl=0.4,
        bumps="0.3,0.3,0.05,1", noise=1e-3, noise_seed=1, crit="none")))
    # 2: 2D active AMR, 16x16 patches, max depth 5, gradient criterion, re-mesh
    #    every 10 steps, two seeded bumps (sigma 0.02-0.06, amplitude 0.5-2).
    #    Shortened to 300 steps so the fixture stays small.
    b2 = seeded_bumps(2, 2, seed=2)
    print(scenario_run("config2_amr_2d", "2d16h1", 2, 16, 1, dict(
        init_levels=2, steps=300, remesh=10, vel="1,0.5", cfl=0.4,
        bumps=",".join(map(str, b2)), noise=1e-3, noise_seed=2, crit="grad",
        rthr=0.05, cthr=0.01, min_level=1, max_level=5), state_every=15))
    # 3: 3D AMR, 8^3 patches, max depth 4, four seeded blobs, v = (1, 0.7, 0.3).
    b3 = seeded_bumps(3, 4, seed=3, sigma=(0.05, 0.08))
    print(scenario_run("config3_amr_3d", "3d8h1", 3, 8, 1, dict(
        init_levels=1, steps=40, remesh=10, vel="1,0.7,0.3", cfl=0.4,
        bumps=",".join(map(str, b3)), noise=0, crit="grad",
        rthr=0.05, cthr=0.01, min_level=1, max_level=3)))
    # Random-flag tree cycles: balance, fragment/recombine, compaction, sort,
    # inter-grid transfer and halo exchange on irregular 2:1 trees.
    print(scenario_tree("tree_random_2d_n4", "2d4h1", 2, 4, 1, dict(
        seed=11, passes=8, init_levels=2, max_level=6, min_level=1, p_refine=0.2, p_coarsen=0.5),
        keep_states={0, 1, 2, 7}))
    print(scenario_tree("tree_random_2d_n8", "2d8h1", 2, 8, 1, dict(
        seed=12, passes=6, init_levels=1, max_level=5, min_level=1, p_refine=0.3, p_coarsen=0.4),
        keep_states={5}))
    print(scenario_tree("tree_random_3d_n4", "3d4h1", 3, 4, 1, dict(
        seed=13, passes=5, init_levels=1, max_level=4, min_level=1, p_refine=0.25, p_coarsen=0.5),
        keep_states={0, 4}))
    print(scenario_tree("tree_random_2d_h2", "2d10h2", 2, 10, 2, dict(
        seed=14, passes=4, init_levels=1, max_level=4, min_level=1, p_refine=0.3, p_coarsen=0.5)))
    for sc in EULER_SCENARIOS:
        print(scenario_euler(*sc))
    print(vtk_golden())


if __name__ == "__main__":
    main()
