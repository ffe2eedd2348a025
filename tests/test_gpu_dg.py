"""The CUDA DG path (amr_tree_dg_advance) against the reference's DG patch
solver (golden fixtures, bit for bit) and against the numpy restatement on
larger uniform trees; argument checks."""
import hashlib

import numpy as np
import pytest

from oracle import dg_oracle as G
from dg_cases import CASES, EULER_CASES, fields_to_leaves, leaves_to_fields, load, printer_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def amr():
    import amr_gb300 as A

    A.lib()
    return A


def _loop_time(dts, next_dt):
    """The time of the reference's DG loop (solver.hpp:125-134) after the
    fixture's steps: each step first takes dt = min(dt, dt_min), then adds
    that updated dt, so the sizes of steps 2..K and the next step's size."""
    t = 0.0
    for d in list(dts[2:]) + [next_dt]:
        t += float(d)
    return t


def _dg_tree(amr, level):
    t = amr.Tree(2, 4, 1, 6, capacity=(1 << (2 * level)) + 64, dtype=amr.F64, fields=16)
    t.refine_uniform(level)
    return t


@pytest.mark.parametrize("name", CASES)
def test_gpu_dg_matches_reference(amr, name):
    z = load(name)
    L = int(z["level"])
    st, dts = z["state"], z["dt"]
    t = _dg_tree(amr, L)
    np.testing.assert_array_equal(t.ids(), z["ids"])
    t.upload_state(leaves_to_fields(st[0]))
    dt, time = float(dts[1]), 0.0
    for k in range(1, len(st)):
        assert dt == dts[k]
        dt, time = t.dg_advance(1, dt, time)
        np.testing.assert_array_equal(fields_to_leaves(t.download_state()), st[k])
    assert time == _loop_time(dts, dt)


@pytest.mark.parametrize("level,steps", [(4, 12), (5, 6)])
def test_gpu_dg_matches_oracle(amr, level, steps):
    U0 = G.initial_state(level)
    t = _dg_tree(amr, level)
    t.upload_state(leaves_to_fields(G.to_leaves(U0, level)))
    dt, time = t.dg_advance(steps, 0.01)
    outs, dts = G.run(level, steps, dt0=0.01, U=U0)
    np.testing.assert_array_equal(fields_to_leaves(t.download_state()), G.to_leaves(outs[-1], level))
    assert dt == min(dts[-1], (1.0 / (2 ** 2 + 1.0)) * 0.5 * ((1.0 / (1 << level)) / 4) / 1.0)


def test_gpu_dg_rejects_other_trees(amr):
    t = amr.Tree(2, 8, 1, 5, capacity=64, dtype=amr.F64, fields=16)
    with pytest.raises(amr.AmrError):
        t.dg_advance(1, 0.01)
    t = amr.Tree(2, 4, 1, 6, capacity=64, dtype=amr.F64, fields=4)
    with pytest.raises(amr.AmrError):
        t.dg_advance(1, 0.01)
    t = _dg_tree(amr, 1)
    with pytest.raises(amr.AmrError):
        t.dg_advance(1, 0.0)


@pytest.mark.parametrize("name", ["dg_amr_l3", "dg_amr_l4"])
def test_gpu_dg_remesh_matches_reference(amr, name):
    """The DG solver loop with its re-mesh (gradient indicator, polynomial
    prolongation and restriction, DG halo across coarse-fine faces) against
    the reference run: leaves and interior states after every step, bit for
    bit."""
    z = load(name)
    L, every, steps = int(z["level"]), int(z["amr"]), int(z["steps"])
    dts = z["dt"]
    t = amr.Tree(2, 4, 1, 6, capacity=8000, dtype=amr.F64, fields=16)
    t.refine_uniform(L)
    np.testing.assert_array_equal(t.ids(), z["ids_0"])
    t.upload_state(leaves_to_fields(z["state_0"]))
    dt, time, next_amr = float(dts[1]), 0.0, 0
    for k in range(1, steps + 1):
        assert dt == dts[k]
        dt, time = t.dg_advance(1, dt, time)
        if k >= next_amr:
            t.dg_remesh(float(z["rthr"]), float(z["cthr"]))
            next_amr = k + every
        np.testing.assert_array_equal(t.ids(), z[f"ids_{k}"])
        np.testing.assert_array_equal(fields_to_leaves(t.download_state()), z[f"state_{k}"])


@pytest.mark.parametrize("equation", ["advection", "euler"])
def test_gpu_dg_run_equals_the_stepwise_loop(amr, equation):
    """amr_tree_dg_run (the solver loop in one call) against the same loop
    driven step by step through amr_tree_dg_advance and amr_tree_dg_remesh:
    same steps, re-meshes, leaves and states."""
    U0 = G.initial_state(3) if equation == "advection" else G.euler_initial_state(3)
    rthr, cthr = (0.05, 0.01) if equation == "advection" else (0.002, 0.0005)
    dt0 = 0.01 if equation == "advection" else 0.002
    a = amr.Tree(2, 4, 1, 6, capacity=8000, dtype=amr.F64, fields=16)
    b = amr.Tree(2, 4, 1, 6, capacity=8000, dtype=amr.F64, fields=16)
    for t in (a, b):
        t.dg_set_equation(equation)
        t.refine_uniform(3)
        t.upload_state(leaves_to_fields(G.to_leaves(U0, 3)))
    st = a.dg_run(dt0, 0.05, 3, rthr, cthr)
    dt, time, step, next_amr, cells, remeshes = dt0, 0.0, 0, 0, 0, 0
    while time < 0.05:
        cells += b.size * 16
        dt, time = b.dg_advance(1, dt, time)
        step += 1
        if step >= next_amr:
            b.dg_remesh(rthr, cthr)
            remeshes += 1
            next_amr = step + 3
    assert (st["steps"], st["remeshes"], st["cells"]) == (step, remeshes, cells)
    assert st["time"] == time and st["next_dt"] == dt
    np.testing.assert_array_equal(a.ids(), b.ids())
    np.testing.assert_array_equal(a.download_state(), b.download_state())


@pytest.mark.parametrize("name", EULER_CASES)
def test_gpu_dg_euler_matches_reference(amr, name):
    """DG Euler (flux, pressure, the patch's running maximum of the face
    speeds, the CFL step reduced on the device) against the reference's DG
    Euler solver: states and step sizes after every step, bit for bit."""
    z = load(name)
    L = int(z["level"])
    st, dts = z["state"], z["dt"]
    t = _dg_tree(amr, L)
    t.dg_set_equation("euler")
    t.upload_state(leaves_to_fields(st[0]))
    dt, time = float(dts[1]), 0.0
    for k in range(1, len(st)):
        assert dt == dts[k]
        dt, time = t.dg_advance(1, dt, time)
        np.testing.assert_array_equal(fields_to_leaves(t.download_state()), st[k])
    assert dts[2] < dts[1]
    assert time == _loop_time(dts, dt)


def test_gpu_dg_euler_remesh_matches_reference(amr):
    """DG Euler with the solver's re-mesh (coarsening of the flat regions,
    refinement along the density front) against the reference run."""
    z = load("dg_euler_amr_l3")
    L, every, steps = int(z["level"]), int(z["amr"]), int(z["steps"])
    dts = z["dt"]
    t = amr.Tree(2, 4, 1, 6, capacity=8000, dtype=amr.F64, fields=16)
    t.dg_set_equation(amr.DG_EULER)
    t.refine_uniform(L)
    t.upload_state(leaves_to_fields(z["state_0"]))
    dt, time, next_amr = float(dts[1]), 0.0, 0
    for k in range(1, steps + 1):
        assert dt == dts[k]
        dt, time = t.dg_advance(1, dt, time)
        if k >= next_amr:
            t.dg_remesh(float(z["rthr"]), float(z["cthr"]))
            next_amr = k + every
        np.testing.assert_array_equal(t.ids(), z[f"ids_{k}"])
        np.testing.assert_array_equal(fields_to_leaves(t.download_state()), z[f"state_{k}"])


def test_gpu_dg_euler_matches_oracle(amr):
    """A larger uniform tree (level 5, 1024 leaves, several steps in one
    call) against the numpy restatement: final state, step size and time."""
    L, steps = 5, 4
    U0 = G.euler_initial_state(L)
    t = _dg_tree(amr, L)
    t.dg_set_equation("euler")
    t.upload_state(leaves_to_fields(G.to_leaves(U0, L)))
    dt, time = t.dg_advance(steps, 0.003)
    outs, dts = G.run(L, steps + 1, dt0=0.003, U=U0, equation="euler")
    np.testing.assert_array_equal(fields_to_leaves(t.download_state()), G.to_leaves(outs[steps - 1], L))
    assert dt == dts[steps]
    assert time == ((((0.0 + dts[1]) + dts[2]) + dts[3]) + dts[4])  # the updated steps, as the loop adds them


def test_gpu_dg_set_equation_rejects_unknown(amr):
    t = _dg_tree(amr, 1)
    with pytest.raises(amr.AmrError):
        amr.check(amr.lib().amr_tree_dg_set_equation(t._h, 7))


@pytest.mark.endtoend
def test_gpu_dg_run_matches_the_reference_main_loop(amr):
    """amr_tree_dg_run against the reference's whole DG main loop
    (DGSolver::run to t = 1 from a uniform level-5 start, re-mesh every 20
    steps, thresholds 0.05 / 0.01; run on the CPU by the reference's own
    code): the step and re-mesh counts, processed cells, largest leaf count,
    final time and next step size, the final leaves, and the final interior
    state bit for bit (its SHA-256)."""
    z = load("dg_main_loop")
    L = int(z["level"])
    t = amr.Tree(2, 4, 1, 6, capacity=8192, dtype=amr.F64, fields=16)
    t.refine_uniform(L)
    t.upload_state(leaves_to_fields(G.to_leaves(G.initial_state(L), L)))
    st = t.dg_run(float(z["dt0"]), float(z["end"]), int(z["amr"]), float(z["rthr"]), float(z["cthr"]))
    assert (st["steps"], st["remeshes"], st["cells"], st["leaves_max"]) == (
        int(z["steps"]), int(z["remeshes"]), int(z["cells"]), int(z["leaves_max"]))
    assert st["time"] == float(z["time"]) and st["next_dt"] == float(z["next_dt"])
    np.testing.assert_array_equal(t.ids(), z["ids"])
    final = np.ascontiguousarray(fields_to_leaves(t.download_state()), dtype="<f8")
    assert final.sum() == float(z["state_sum"])
    assert hashlib.sha256(final.tobytes()).hexdigest() == str(z["state_sha256"])


def _fixture_tree_on_gpu(amr, name, dump):
    """The tree of dump `dump` of a DG fixture on the device: the uniform
    level, or the fixture's re-mesh loop replayed to that dump, then the
    fixture's state of that dump uploaded."""
    z = load(name)
    L = int(z["level"])
    t = amr.Tree(2, 4, 1, 6, capacity=8000, dtype=amr.F64, fields=16)
    t.dg_set_equation(str(z["equation"]))
    t.refine_uniform(L)
    if "state" in z:
        t.upload_state(leaves_to_fields(z["state"][dump]))
        return t
    every, dts = int(z["amr"]), z["dt"]
    t.upload_state(leaves_to_fields(z["state_0"]))
    dt, time, next_amr = float(dts[1]), 0.0, 0
    for k in range(1, dump + 1):
        dt, time = t.dg_advance(1, dt, time)
        if k >= next_amr:
            t.dg_remesh(float(z["rthr"]), float(z["cthr"]))
            next_amr = k + every
    np.testing.assert_array_equal(t.ids(), z[f"ids_{dump}"])
    t.upload_state(leaves_to_fields(z[f"state_{dump}"]))
    return t


@pytest.mark.endtoend
@pytest.mark.parametrize("name", sorted(printer_cases()))
def test_gpu_dg_printer_matches_reference(amr, name, tmp_path):
    """amr_tree_dg_write_vtk against the file the reference's
    dg_tree_printer_2d wrote for the same tree and state: byte for byte
    (SHA-256 and length)."""
    c = printer_cases()[name]
    t = _fixture_tree_on_gpu(amr, c["fixture"], c["dump"])
    path = tmp_path / f"{name}.vtk"
    t.dg_write_vtk(path)
    b = path.read_bytes()
    assert len(b) == c["bytes"] and hashlib.sha256(b).hexdigest() == c["sha256"]


def test_gpu_dg_printer_rejects_other_trees(amr, tmp_path):
    t = amr.Tree(2, 8, 1, 5, capacity=64, dtype=amr.F64, fields=16)
    with pytest.raises(amr.AmrError):
        t.dg_write_vtk(tmp_path / "x.vtk")
