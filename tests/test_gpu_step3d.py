"""The staged 3D update (k_step3d: one warp per 8^3 or 4^3 patch, bulk-copied
tiles, upwind ghost faces by the halo rules) on trees above the cluster
kernel's leaf limit, where runs go through graph intervals (k_run_step3d)
and the host loop through advance (k_step3d).

Bars: graph run == host-driven loop bit for bit (FP64 and FP32: the same
update arithmetic in both kernels); FP64 against the oracle, trees and
neighbour-derived flags bit-exact and states within 1e-12 relative L2; FP32
against the FP64 oracle within 1e-5 per re-mesh interval while the trees
agree."""
import numpy as np
import pytest

from conftest import interior, rel_l2

pytestmark = pytest.mark.gpu

VEL, CFL = (1.0, 0.7, 0.3), 0.4
RTHR, CTHR, MINL, MAXL = 0.05, 0.01, 3, 5
STEPS, INTERVAL, DEPTH = 20, 10, 6


@pytest.fixture(scope="module")
def amr():
    import amr_gb300 as A

    A.lib()
    return A


def _tree(A, n, dtype, level=4):
    b = A.seeded_bumps(3, 4, 3, sigma=(0.05, 0.08))
    t = A.Tree(3, n, 1, DEPTH, capacity=40000, dtype=dtype)
    t.refine_uniform(level)  # 4096 leaves: above the cluster kernel's limit
    t.upload_state(A.gaussian_state(t.ids(), 3, n, 1, DEPTH, b))
    t.halo_exchange()
    return t


def _host_loop(t):
    done, sum_dt = 0, 0.0
    while done < STEPS:
        t.advance(min(INTERVAL, STEPS - done), VEL, CFL)
        acc, ex = t.finish_advance()
        done += ex
        sum_dt += acc
        t.flags_gradient(RTHR, CTHR, MINL, MAXL)
        t.remesh()
    return sum_dt, done


@pytest.mark.parametrize("n", [8, 4])
@pytest.mark.parametrize("prec", ["F64", "F32"])
def test_graph_run_equals_host_loop(amr, n, prec):
    dtype = getattr(amr, prec)
    a = _tree(amr, n, dtype)
    st = a.run(STEPS, INTERVAL, VEL, CFL, "grad", RTHR, CTHR, MINL, MAXL)
    assert st["graph_intervals"] == STEPS // INTERVAL and st["persistent_intervals"] == 0
    assert st["remeshes_changed"] > 0  # the tree adapts
    b = _tree(amr, n, dtype)
    sum_dt, done = _host_loop(b)
    assert (st["sum_dt"], st["executed_steps"]) == (sum_dt, done)
    np.testing.assert_array_equal(a.ids(), b.ids())
    np.testing.assert_array_equal(interior(a.download_state(), 3, n, 1), interior(b.download_state(), 3, n, 1))


@pytest.mark.parametrize("prec,tol", [("F64", 1e-12), ("F32", 1e-5)])
def test_against_oracle(amr, oracle_mod, prec, tol):
    O = oracle_mod
    O.set_threads(16)
    n = 8
    t = _tree(amr, n, getattr(amr, prec))
    o = O.OracleTree(3, n, 1, DEPTH, 40000)
    o.refine_all(4)
    np.testing.assert_array_equal(t.ids(), o.ids())
    o.set_state(t.download_state().astype(np.float64))
    o.halo_exchange()
    done = 0
    while done < STEPS:
        k = min(INTERVAL, STEPS - done)
        t.advance(k, VEL, CFL)
        acc_t, ex = t.finish_advance()
        acc_o, _ = o.advance(k, VEL, CFL)
        assert acc_t == acc_o
        done += ex
        assert rel_l2(interior(t.download_state(), 3, n, 1), interior(o.state(), 3, n, 1)) <= tol
        fo = o.flags_gradient(RTHR, CTHR, MINL, MAXL)
        t.flags_gradient(RTHR, CTHR, MINL, MAXL)
        np.testing.assert_array_equal(t.get_flags(), fo)
        assert o.reconstruct(fo) == 0
        o.halo_exchange()
        t.remesh()
        np.testing.assert_array_equal(t.ids(), o.ids())


FOREST = dict(caps=[1, 2, 1, 2, 2], bounds=[(1, 2), (1, 3), (0, 2), (2, 3), (1, 2)],
              vels=[(1.0, 0.7, 0.3), (-0.6, 0.4, -0.8), (0.0, -1.0, 0.5), (0.3, 0.0, 0.0), (-0.2, -0.9, -0.4)])


@pytest.mark.parametrize("n", [8, 4])
def test_forest_per_instance_velocities_against_oracle(amr, oracle_mod, n):
    """A 3D forest whose instances move in different directions (signs of
    every component, zero components): the staged kernel takes each leaf's
    upwind sides from its instance; per instance the trees equal the oracle's
    and the FP64 states agree within 1e-12; the graph run equals the
    step-by-step calls bit for bit."""
    O = oracle_mod
    c = FOREST
    K = len(c["caps"])
    oracle, init = [], []
    for i, cap in enumerate(c["caps"]):
        o = O.OracleTree(3, n, 1, 4, 20000)
        o.refine_all(cap)
        o.init_state(amr.seeded_bumps(3, 2, 200 + i, sigma=(0.08, 0.15)), 1e-3, i + 1)
        o.halo_exchange()
        init.append(o.state())
        oracle.append(o)

    def forest():
        f = amr.Tree(3, n, 1, 4, capacity=20000, instances=K)
        f.refine_to_levels(c["caps"])
        f.upload_state(np.concatenate(init))
        f.set_instance_params(velocity=c["vels"], level_bounds=c["bounds"])
        return f

    a, b = forest(), forest()
    a.run(STEPS, INTERVAL, None, CFL, "grad", RTHR, CTHR)
    for _ in range(STEPS // INTERVAL):
        b.advance(INTERVAL, None, CFL)
        b.finish_advance()
        b.flags_gradient(RTHR, CTHR, 0, 0)  # per-instance bounds apply
        b.remesh()
    np.testing.assert_array_equal(a.ids(), b.ids())
    np.testing.assert_array_equal(interior(a.download_state(), 3, n, 1), interior(b.download_state(), 3, n, 1))
    for i, o in enumerate(oracle):
        for _ in range(STEPS // INTERVAL):
            o.advance(INTERVAL, c["vels"][i], CFL)
            assert o.reconstruct(o.flags_gradient(RTHR, CTHR, *c["bounds"][i])) == 0
            o.halo_exchange()
    off = a.instance_offsets()
    ids = a.ids() & np.uint64((1 << (6 + 3 * 4)) - 1)
    st = interior(a.download_state(), 3, n, 1)
    for i, o in enumerate(oracle):
        np.testing.assert_array_equal(ids[off[i]:off[i + 1]], o.ids())
        assert rel_l2(st[off[i]:off[i + 1]], interior(o.state(), 3, n, 1)) <= 1e-12, i


_SHAPE_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import amr_gb300 as A
b = A.seeded_bumps(3, 4, 3, sigma=(0.05, 0.08))
out = []
for n in (8, 4):
    for dt in (A.F64, A.F32):
        t = A.Tree(3, n, 1, 6, capacity=5000, dtype=dt)
        t.refine_uniform(3)
        t.upload_state(A.gaussian_state(t.ids(), 3, n, 1, 6, b))
        t.advance(12, (1.0, -0.7, 0.3), 0.4)
        t.finish_advance()
        out.append(t.download_state().astype(np.float64).ravel())
np.save(sys.argv[2], np.concatenate(out))
"""


def test_launch_shapes_agree(tmp_path):
    """Every built (warps per block, ring depth) pair of the staged 3D kernel
    (AMR_GB300_STEP3D, read once per process) gives the same states bit for
    bit, in FP64 and FP32, for 8^3 and 4^3 patches (each in its own process)."""
    import os
    import subprocess
    import sys
    from pathlib import Path

    pkg = str(Path(__file__).resolve().parents[1] / "gpu-amr_gb300")
    res = {}
    for shape in ("", "4,2", "4,3", "8,2", "8,3"):
        env = dict(os.environ)
        env.pop("AMR_GB300_STEP3D", None)
        if shape:
            env["AMR_GB300_STEP3D"] = shape
        out = tmp_path / f"s{shape.replace(',', '_') or 'default'}.npy"
        subprocess.run([sys.executable, "-c", _SHAPE_SCRIPT, pkg, str(out)], env=env, check=True, timeout=600)
        res[shape] = np.load(out)
    ref = res[""]
    for shape, v in res.items():
        np.testing.assert_array_equal(v, ref, err_msg=shape)
