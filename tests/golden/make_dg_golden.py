"""Generate the DG golden fixtures in this folder from the REAL reference.

Builds oracle/_ref/ref_dg_driver and ref_dg_euler_driver (the unmodified
reference DG patch solver, include/dg_helpers, compiled by oracle/Makefile,
the second with the reference's DG Euler equations in place of advection;
needs the reference checkout, so this runs only where it is present) and
records each scenario as a compressed .npz:

  ids            Morton ids of the leaves (uniform level, Morton order)
  state          [dump, leaf, cell, node, variable] interior nodal values;
                 dump 0 is the initial state, dump k the state after step k
  dt             [dump] step size used to reach each dump (0 for dump 0)
  with re-mesh:  ids_k / state_k per dump k (the leaf count changes), and
                 amr (interval), rthr, cthr
  main loop:     dg_main_loop.npz, the reference's DGSolver::run loop to
                 t = 1 (the example's configuration): the final leaves,
                 the SHA-256 of the final interior state ([leaf, cell, node,
                 variable] little-endian float64) and the loop's counts

Usage:  python tests/golden/make_dg_golden.py              (every fixture)
        python tests/golden/make_dg_golden.py main_loop    (dg_main_loop.npz only)
"""
from __future__ import annotations

import struct
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
DRIVERS = {"advection": REPO / "oracle" / "_ref" / "ref_dg_driver",
           "euler": REPO / "oracle" / "_ref" / "ref_dg_euler_driver"}

SCENARIOS = {
    # name: (level, steps, initial dt, re-mesh interval (0: none), refine / coarsen thresholds, equation)
    "dg_advection_l2": (2, 3, 0.01, 0, 0.05, 0.01, "advection"),
    "dg_advection_l3": (3, 4, 0.01, 0, 0.05, 0.01, "advection"),
    "dg_advection_l3_small_dt": (3, 3, 0.001, 0, 0.05, 0.01, "advection"),
    # with the DG solver's re-mesh after steps 1, 3 (and 5): refinement to levels
    # 4-5 (the reference's thresholds) ...
    "dg_amr_l3": (3, 4, 0.01, 2, 0.05, 0.01, "advection"),
    # ... and refinement to level 6 followed by coarsening back to level 5
    "dg_amr_l4": (4, 6, 0.001, 2, 0.05, 0.03, "advection"),
    # Euler pressure pulse: the first step size above the CFL step, which
    # the patches' wave speeds then set ...
    "dg_euler_l3": (3, 5, 0.003, 0, 0.05, 0.01, "euler"),
    # ... and with re-mesh: coarsening of the flat regions (64 -> 40 leaves),
    # then refinement along the density front (136, 388 leaves)
    "dg_euler_amr_l3": (3, 5, 0.002, 2, 0.002, 0.0005, "euler"),
}


# the reference's DG main loop: level, initial dt, re-mesh interval,
# thresholds, end time
MAIN_LOOP = (5, 0.01, 20, 0.05, 0.01, 1.0)


def main_loop():
    """Run DGSolver::run's loop (CPU, about ten minutes) and record it.  The
    run starts from the reference's initial state, which the numpy
    restatement reproduces bit for bit at this level (checked here), so a
    test can start from the restatement's."""
    import hashlib
    import sys

    sys.path.insert(0, str(REPO))
    from oracle import dg_oracle as G

    level, dt0, amr, rthr, cthr, end = MAIN_LOOP
    init = Path("/tmp") / "dg_main_loop_init.bin"
    subprocess.run([str(DRIVERS["advection"]), f"level={level}", "steps=0", "capacity=8192", f"out={init}"],
                   check=True)
    _, st0, _ = read_dumps(init)
    assert np.array_equal(G.to_leaves(G.initial_state(level), level), st0[0])
    out = Path("/tmp") / "dg_main_loop.bin"
    r = subprocess.run([str(DRIVERS["advection"]), f"level={level}", f"dt0={dt0}", f"amr={amr}", f"rthr={rthr}",
                        f"cthr={cthr}", f"end={end}", "capacity=8192", f"out={out}"],
                       check=True, capture_output=True, text=True)
    steps, remeshes, cells, leaves_max, time, next_dt = r.stdout.split()
    # the driver writes the initial tree first and the tree at the end of the
    # loop last: the record is the last dump
    idss, states, _ = read_dumps_any(out)
    assert len(idss) == 2 and len(idss[0]) == 4 ** level
    final_ids, final = idss[-1], states[-1]
    digest = hashlib.sha256(np.ascontiguousarray(final, dtype="<f8").tobytes()).hexdigest()
    np.savez_compressed(HERE / "dg_main_loop.npz", ids=final_ids, state_sha256=digest, level=level, dt0=dt0, amr=amr,
                        rthr=rthr, cthr=cthr, end=end, steps=int(steps), remeshes=int(remeshes), cells=int(cells),
                        leaves_max=int(leaves_max), time=float(time), next_dt=float(next_dt),
                        state_sum=float(final.sum()))
    print("dg_main_loop", steps, remeshes, cells, leaves_max, time, next_dt, len(final_ids))


# the reference's DG printer on fixture trees: name -> (fixture, dump, driver,
# driver arguments reproducing that dump as the final tree)
PRINTS = {
    "dg_vtk_l2": ("dg_advection_l2", 0, "advection", ["level=2", "steps=0"]),
    "dg_vtk_amr_l3": ("dg_amr_l3", 4, "advection",
                      ["level=3", "steps=4", "dt0=0.01", "amr=2", "rthr=0.05", "cthr=0.01"]),
    "dg_vtk_euler_amr_l3": ("dg_euler_amr_l3", 5, "euler",
                            ["level=3", "steps=5", "dt0=0.002", "amr=2", "rthr=0.002", "cthr=0.0005"]),
}


def printer_golden():
    """SHA-256 and length of the reference printer's file for each PRINTS
    entry (dg_vtk.json); the driver runs in a scratch folder because the
    printer clears ./vtk_output."""
    import hashlib
    import json

    work = Path("/tmp") / "dg_vtk_golden"
    work.mkdir(exist_ok=True)
    rec = {}
    for name, (fixture, dump, eq, dargs) in PRINTS.items():
        vtk = work / f"{name}.vtk"
        subprocess.run([str(DRIVERS[eq]), *dargs, "capacity=8000", f"out={work / 'dump.bin'}", f"vtk={vtk}"],
                       check=True, cwd=work)
        b = vtk.read_bytes()
        rec[name] = {"fixture": fixture, "dump": dump, "sha256": hashlib.sha256(b).hexdigest(), "bytes": len(b)}
    (HERE / "dg_vtk.json").write_text(json.dumps(rec, indent=1) + "\n")
    print("dg_vtk", {k: v["bytes"] for k, v in rec.items()})


def read_dumps_any(path: Path):
    """The dumps of a file whose first record may carry any step number."""
    b = path.read_bytes()
    assert b[:4] == b"DGS1"
    o = 4
    idss, states = [], []
    while o < len(b):
        o += 12
        P, = struct.unpack_from("<Q", b, o)
        o += 8
        idss.append(np.frombuffer(b, np.uint64, P, o).copy())
        o += 8 * P
        states.append(np.frombuffer(b, np.float64, P * 256, o).reshape(P, 16, 4, 4).copy())
        o += 8 * P * 256
    return idss, states, None


def read_dumps(path: Path):
    b = path.read_bytes()
    assert b[:4] == b"DGS1"
    o = 4
    idss, states, dts = [], [], []
    while o < len(b):
        step, = struct.unpack_from("<I", b, o)
        o += 4
        dt, = struct.unpack_from("<d", b, o)
        o += 8
        P, = struct.unpack_from("<Q", b, o)
        o += 8
        ids = np.frombuffer(b, np.uint64, P, o).copy()
        o += 8 * P
        st = np.frombuffer(b, np.float64, P * 16 * 4 * 4, o).reshape(P, 16, 4, 4).copy()
        o += 8 * P * 256
        assert step == len(states)
        idss.append(ids)
        states.append(st)
        dts.append(dt)
    return idss, states, np.array(dts)


def main():
    import sys

    subprocess.run(["make", "-C", str(REPO / "oracle"), "ref"], check=True)
    if sys.argv[1:] == ["main_loop"]:
        main_loop()
        return
    for name, (level, steps, dt0, amr, rthr, cthr, eq) in SCENARIOS.items():
        out = Path("/tmp") / f"{name}.bin"
        subprocess.run([str(DRIVERS[eq]), f"level={level}", f"steps={steps}", f"dt0={dt0}", f"amr={amr}",
                        f"rthr={rthr}", f"cthr={cthr}", "capacity=8000", f"out={out}"], check=True)
        idss, states, dts = read_dumps(out)
        if amr == 0:
            np.savez_compressed(HERE / f"{name}.npz", ids=idss[0], state=np.stack(states), dt=dts, level=level,
                                equation=eq)
        else:
            extra = {f"ids_{k}": v for k, v in enumerate(idss)}
            extra.update({f"state_{k}": v for k, v in enumerate(states)})
            np.savez_compressed(HERE / f"{name}.npz", dt=dts, level=level, amr=amr, rthr=rthr, cthr=cthr,
                                steps=steps, equation=eq, **extra)
        print(name, [len(i) for i in idss], dts)
    printer_golden()
    main_loop()


if __name__ == "__main__":
    main()
