"""The C++ drop-in (gpu-amr_gb300/host: ndtree, amr_solver, morton_id, ...)
compiled against the reference's own solver tests and benchmark loop."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import bumps_of, load_golden, rel_l2

REPO = Path(__file__).resolve().parents[1]
SRC = REPO / "tests" / "cpp" / "dropin_tests.cpp"
FLAGS = ["-std=c++20", "-O2", "-I", str(REPO / "include"), "-I", str(REPO / "gpu-amr_gb300" / "host")]


def test_dropin_headers_compile():
    subprocess.run(["g++", *FLAGS, "-fsyntax-only", str(SRC)], check=True)


@pytest.fixture(scope="module")
def dropin_exe(tmp_path_factory):
    import __graft_entry__ as g

    lib = g.build_library()
    exe = tmp_path_factory.mktemp("cpp") / "dropin_tests"
    subprocess.run(["g++", *FLAGS, str(SRC), "-o", str(exe), "-L", str(lib.parent), "-lamr_gb300",
                    f"-Wl,-rpath,{lib.parent}"], check=True)
    return exe


@pytest.mark.gpu
def test_reference_solver_tests_pass_on_dropin(dropin_exe):
    """PulseCenterMovement / PulseCenterMovementAMR of the reference
    (tests/advection_equation_amr.t.cpp:50-232), 10x10 and 50x50 patches."""
    r = subprocess.run([str(dropin_exe), "tests"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASSED" in r.stdout


@pytest.mark.gpu
def test_benchmark_loop_through_dropin_matches_reference(dropin_exe):
    z, meta = load_golden("config2_amr_2d")
    p = meta["params"]
    b = bumps_of(meta)
    args = [str(dropin_exe), "bench", str(p["steps"]), str(p["remesh"]), str(p["noise"]), str(p["noise_seed"])]
    args += [repr(float(v)) for v in b]
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    head = lines[0].split()
    sum_dt, steps = float(head[1]), int(head[3])
    ids = np.array([int(l.split()[1]) for l in lines if l.startswith("id ")], np.uint64)
    u = np.array([float(l.split()[1]) for l in lines if l.startswith("u ")])
    assert steps == int(z["steps"]) and sum_dt == float(z["sum_dt"])
    np.testing.assert_array_equal(ids, z["final_ids"])
    assert rel_l2(u, z["state_final"].reshape(-1)) <= 1e-12


@pytest.mark.gpu
def test_adjoint_through_cpp_header(dropin_exe):
    """amr::gb300::adjoint (solver/adjoint.hpp): dot-product identity of the
    discrete adjoint on a 2:1 mesh, host buffers."""
    r = subprocess.run([str(dropin_exe), "adjoint"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASSED" in r.stdout


@pytest.mark.gpu
def test_euler_benchmark_through_dropin_matches_reference(dropin_exe):
    """The Euler benchmark's set-up and loop written against the reference's
    API (amr_solver<..., EulerPhysics2D, 2>, initialize, host max-Rho
    criterion through reconstruct_tree) on the 2D Euler fixture's
    configuration: initial state, trees, final state of every field
    (interior and face-ghost cells) and the simulated time equal the
    reference's run.  The initial condition goes through the host's exp; if
    that differs from the fixture machine's in a last bit, the bars fall
    back to 1e-12 relative."""
    from conftest import face_mask

    z, meta = load_golden("euler_pulse_2d")
    p = meta["params"]
    args = [str(dropin_exe), "euler", str(p["steps"]), str(p["remesh"]), str(p["init_levels"]),
            str(p["min_level"]), str(p["max_level"])]
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    s0 = np.array([float(l.split()[1]) for l in lines if l.startswith("s0 ")])
    s1 = np.array([float(l.split()[1]) for l in lines if l.startswith("s1 ")])
    head = [l for l in lines if l.startswith("time ")][0].split()
    time, steps = float(head[1]), int(head[3])
    ids = np.array([int(l.split()[1]) for l in lines if l.startswith("id ")], np.uint64)
    m = face_mask(2, 8, 1)
    want0 = np.moveaxis(z["state_init"], 1, 0)[..., m].ravel()
    want1 = np.moveaxis(z["state_final"], 1, 0)[..., m].ravel()
    k = int(z["remeshes"]) - 1
    np.testing.assert_array_equal(ids, z[f"ids_{k}"])
    assert steps == int(z["steps"])
    if np.array_equal(s0, want0):
        np.testing.assert_array_equal(s1, want1)
        assert time == float(z["time"])
    else:
        assert rel_l2(s0, want0) <= 1e-15
        assert rel_l2(s1, want1) <= 1e-12 and abs(time - float(z["time"])) <= 1e-12 * float(z["time"])


DG_SRC = REPO / "tests" / "cpp" / "dg_dropin.cpp"


def test_dg_dropin_headers_compile():
    """dg_helpers/solver.hpp and config/generated_config.hpp (the reference's
    DG solver API) compile with a program written like the reference's DG
    example."""
    subprocess.run(["g++", *FLAGS, "-fsyntax-only", str(DG_SRC)], check=True)


def _read_trees(path):
    raw = path.read_bytes()
    out, o = [], 0
    while o < len(raw):
        P = int(np.frombuffer(raw, np.uint64, 1, o)[0])
        o += 8
        ids = np.frombuffer(raw, np.uint64, P, o).copy()
        o += 8 * P
        state = np.frombuffer(raw, np.float64, 16 * P * 36, o).reshape(16, P, 6, 6).copy()
        o += 8 * 16 * P * 36
        out.append((ids, state))
    return out


@pytest.mark.gpu
@pytest.mark.endtoend
def test_dg_solver_through_cpp_header_equals_dg_run(tmp_path):
    """DGSolver<Policy>::run() of the C++ header (level-5 start, initial dt
    0.01, re-mesh every 20 steps, output every 0.01, to t = 0.05) against
    amr_tree_dg_run from the same initial state: processed cells, final
    leaves and interior states bit for bit; one VTK file at time 0 and one
    per plot time reached.  The header's initial values (the equation's
    initial condition at the nodes, through the host's sin) agree with the
    numpy restatement's to 4 ulp."""
    import __graft_entry__ as g
    import amr_gb300 as A
    from dg_cases import fields_to_leaves
    from oracle import dg_oracle as G

    lib = g.build_library()
    exe = tmp_path / "dg_dropin"
    subprocess.run(["g++", *FLAGS, str(DG_SRC), "-o", str(exe), "-L", str(lib.parent), "-lamr_gb300",
                    f"-Wl,-rpath,{lib.parent}"], check=True)
    r = subprocess.run([str(exe), str(tmp_path / "trees.bin")], capture_output=True, text=True, timeout=600,
                       cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    words = r.stdout.split()
    processed, files = int(words[1]), int(words[3])
    (ids0, s0), (ids1, s1) = _read_trees(tmp_path / "trees.bin")
    np.testing.assert_allclose(fields_to_leaves(s0), G.to_leaves(G.initial_state(5), 5), rtol=4 * 2.0 ** -52,
                               atol=4 * 2.0 ** -52)
    t = A.Tree(2, 4, 1, 6, capacity=8192, dtype=A.F64, fields=16)
    t.refine_uniform(5)
    np.testing.assert_array_equal(t.ids(), ids0)
    t.upload_state(s0)
    st = t.dg_run(0.01, 0.05, 20, 0.05, 0.01)
    assert processed == st["cells"]
    np.testing.assert_array_equal(t.ids(), ids1)
    np.testing.assert_array_equal(fields_to_leaves(t.download_state()), fields_to_leaves(s1))
    assert 5 <= files <= 6


@pytest.mark.parametrize("name", ["dg_advection_l3", "dg_euler_l3"])
def test_dg_dropin_initial_state_matches_reference(name, tmp_path):
    """DGSolver<Policy>::initial_state (the TreeBuilder's nodal initial
    values, host arithmetic only) for the reference's level-3 tree against
    the initial state the reference's own TreeBuilder arithmetic produced
    (dump 0 of the DG fixtures, advection and Euler): bit for bit."""
    from dg_cases import fields_to_leaves, load

    z = load(name)
    ids, st0 = z["ids"], z["state"][0]
    exe = tmp_path / "dg_initial_state"
    subprocess.run(["g++", *FLAGS, str(REPO / "tests" / "cpp" / "dg_initial_state.cpp"), "-o", str(exe)],
                   check=True)
    (tmp_path / "ids.bin").write_bytes(np.ascontiguousarray(ids, dtype=np.uint64).tobytes())
    eq = str(z["equation"])
    subprocess.run([str(exe), eq, str(tmp_path / "ids.bin"), str(tmp_path / "state.bin")], check=True)
    state = np.fromfile(tmp_path / "state.bin", np.float64).reshape(16, len(ids), 6, 6)
    np.testing.assert_array_equal(fields_to_leaves(state), st0)
