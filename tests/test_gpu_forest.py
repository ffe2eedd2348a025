"""Forests (many independent AMR instances in one tree object) and the graph
path of amr_tree_run, through the C ABI, against the oracle.

Each instance of a forest is an independent tree: its leaves, levels,
neighbour tables, time steps and state must equal the oracle run of that
instance alone (the oracle has no notion of a forest).  Bars:
  * Morton ids (instance prefix removed), levels: bit-exact.
  * FP64 interior state: relative L2 <= 1e-12 per instance.
  * Sum of time steps per instance: exact.
  * Graph replay, host-driven launches and the cluster kernel: bit-identical.
  * FP32 forest state against the FP64 oracle: relative L2 <= 1e-5.
"""
import numpy as np
import pytest

from conftest import interior, rel_l2

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-12
FP32_TOL = 1e-5


@pytest.fixture(scope="module")
def amr():
    import amr_gb300 as A

    A.lib()
    return A


def _local(ids, rank, depth):
    return np.asarray(ids, np.uint64) & np.uint64((1 << (6 + rank * depth)) - 1)


def _oracle_instance(O, n, depth, cap, bumps, seed, vel, bounds, steps, interval, cfl, rthr, cthr, crit="grad"):
    """The reference benchmark loop for one instance (refine to its cap,
    Gaussian bumps + seeded noise, advance/flag/re-mesh)."""
    t = O.OracleTree(2, n, 1, depth, 20000)
    t.refine_all(cap)
    t.init_state(bumps, 1e-3, seed)
    t.halo_exchange()
    s0 = t.state()
    done, sum_dt = 0, 0.0
    while done < steps:
        k = min(interval, steps - done)
        acc, ex = t.advance(k, vel, cfl)
        sum_dt += acc
        done += ex
        if crit != "none":
            f = t.flags_gradient(rthr, cthr, bounds[0], bounds[1])
            assert t.reconstruct(f) == 0
            t.halo_exchange()
        if ex == 0:
            break
    return s0, t, sum_dt


CASE = dict(
    n=16,
    depth=5,
    caps=[1, 2, 3, 2, 1, 2],
    bounds=[(0, 2), (1, 3), (2, 4), (1, 2), (0, 3), (2, 2)],
    vels=[(1.0, 0.5), (-0.7, 0.3), (0.2, -1.0), (-0.5, -0.5), (0.0, 0.8), (0.9, 0.0)],
    steps=30,
    interval=10,
    cfl=0.4,
    rthr=0.05,
    cthr=0.01,
)


@pytest.fixture(scope="module")
def oracle_runs(oracle_mod):
    import amr_gb300 as A

    c = CASE
    out = []
    for i, cap in enumerate(c["caps"]):
        bumps = A.seeded_bumps(2, 2, 100 + i, sigma=(0.04, 0.08), amp=(0.5, 2.0))
        out.append(_oracle_instance(oracle_mod, c["n"], c["depth"], cap, bumps, i + 1, c["vels"][i], c["bounds"][i],
                                    c["steps"], c["interval"], c["cfl"], c["rthr"], c["cthr"]))
    return out


def _forest(amr, runs, dtype, capacity=20000):
    c = CASE
    K = len(c["caps"])
    f = amr.Tree(2, c["n"], 1, c["depth"], capacity=capacity, dtype=dtype, instances=K)
    f.refine_to_levels(c["caps"])
    off = f.instance_offsets()
    ids = f.ids()
    for i in range(K):
        np.testing.assert_array_equal(ids[off[i]:off[i + 1]] >> np.uint64(6 + 2 * c["depth"]), i)
        assert off[i + 1] - off[i] == 4 ** c["caps"][i]
    f.upload_state(np.concatenate([r[0] for r in runs]))
    f.set_instance_params(velocity=c["vels"], level_bounds=c["bounds"])
    return f


def _run(f, **kw):
    c = CASE
    return f.run(c["steps"], c["interval"], None, c["cfl"], "grad", c["rthr"], c["cthr"], **kw)


def _check_against_oracle(f, runs, tol):
    c = CASE
    off = f.instance_offsets()
    ids = f.ids()
    lev = f.levels()
    st = interior(f.download_state(), 2, c["n"], 1)
    acc, cnt = f.instance_time()
    for i, (_, o, sum_dt) in enumerate(runs):
        sl = slice(off[i], off[i + 1])
        np.testing.assert_array_equal(_local(ids[sl], 2, c["depth"]), o.ids())
        np.testing.assert_array_equal(lev[sl], (o.ids() & np.uint64(63)).astype(np.int32))
        assert rel_l2(st[sl], interior(o.state(), 2, c["n"], 1)) <= tol, i
        assert acc[i] == sum_dt and cnt[i] == c["steps"]


def test_forest_instances_match_oracle_graph_path(amr, oracle_runs):
    f = _forest(amr, oracle_runs, amr.F64)
    st = _run(f)
    assert st["graph_intervals"] == st["intervals"] == 3 and st["persistent_intervals"] == 0
    assert st["remeshes"] == 3
    _check_against_oracle(f, oracle_runs, STATE_TOL)


def test_forest_graph_equals_host_driven(amr, oracle_runs):
    res = []
    for graph in (True, False):
        f = _forest(amr, oracle_runs, amr.F64)
        st = _run(f, graph=graph)
        assert (st["graph_intervals"] > 0) == graph
        res.append(({k: st[k] for k in ("executed_steps", "cell_updates", "remeshes", "intervals", "leaves_min",
                                        "leaves_max", "leaves_mean")}, f.ids(), f.levels(),
                    interior(f.download_state(), 2, CASE["n"], 1)))
    assert res[0][0] == res[1][0]
    for a, b in zip(res[0][1:], res[1][1:]):
        np.testing.assert_array_equal(a, b)


def test_forest_step_by_step_api(amr, oracle_runs):
    """advance(velocity=None) + flags + remesh per interval == the oracle."""
    c = CASE
    f = _forest(amr, oracle_runs, amr.F64)
    for _ in range(c["steps"] // c["interval"]):
        f.advance(c["interval"], None, c["cfl"])
        f.finish_advance()
        f.flags_gradient(c["rthr"], c["cthr"], 0, 0)  # per-instance bounds apply
        f.remesh()
    off = f.instance_offsets()
    st = interior(f.download_state(), 2, c["n"], 1)
    for i, (_, o, _) in enumerate(oracle_runs):
        np.testing.assert_array_equal(_local(f.ids()[off[i]:off[i + 1]], 2, c["depth"]), o.ids())
        assert rel_l2(st[off[i]:off[i + 1]], interior(o.state(), 2, c["n"], 1)) <= STATE_TOL


def test_fp32_forest_static_caps_against_fp64_oracle(amr, oracle_mod):
    """FP32 state, instances held at their caps (min = max level): the tree
    is the oracle's and the state within 1e-5 relative L2 per instance."""
    import amr_gb300 as A

    c = CASE
    caps = c["caps"]
    runs = []
    for i, cap in enumerate(caps):
        bumps = A.seeded_bumps(2, 2, 200 + i, sigma=(0.04, 0.08), amp=(0.5, 2.0))
        runs.append(_oracle_instance(oracle_mod, c["n"], c["depth"], cap, bumps, i + 7, c["vels"][i], (cap, cap), 40,
                                     10, c["cfl"], c["rthr"], c["cthr"]))
    f = amr.Tree(2, c["n"], 1, c["depth"], capacity=20000, dtype=amr.F32, instances=len(caps))
    f.refine_to_levels(caps)
    f.upload_state(np.concatenate([r[0] for r in runs]).astype(np.float32))
    f.set_instance_params(velocity=c["vels"], level_bounds=[(k, k) for k in caps])
    st = f.run(40, 10, None, c["cfl"], "grad", c["rthr"], c["cthr"])
    assert st["graph_intervals"] == 4
    off = f.instance_offsets()
    s = interior(f.download_state(), 2, c["n"], 1)
    acc, _ = f.instance_time()
    for i, (_, o, sum_dt) in enumerate(runs):
        np.testing.assert_array_equal(_local(f.ids()[off[i]:off[i + 1]], 2, c["depth"]), o.ids())
        assert rel_l2(s[off[i]:off[i + 1]], interior(o.state(), 2, c["n"], 1)) <= FP32_TOL
        assert acc[i] == sum_dt


def test_forest_capacity_error_leaves_consistent_tree(amr, oracle_runs):
    c = CASE
    K = len(c["caps"])
    f = amr.Tree(2, c["n"], 1, c["depth"], capacity=200, dtype=amr.F64, instances=K)
    with pytest.raises(amr.AmrError) as e:
        f.refine_to_levels([3] * K)
    assert e.value.code == amr.AMR_ERR_CAPACITY
    assert f.size == len(f.ids())
    # graph path: every leaf wants to refine, the second re-mesh overflows
    g = amr.Tree(2, c["n"], 1, c["depth"], capacity=6 * 16 + 10, dtype=amr.F64, instances=K)
    g.refine_to_levels([1] * K)
    g.set_instance_params(velocity=c["vels"], level_bounds=[(0, 4)] * K)
    g.upload_state(np.random.default_rng(0).random((g.size, 18, 18)))
    with pytest.raises(amr.AmrError) as e:
        g.run(20, 5, None, 0.4, "grad", 1e-9, 1e-12)
    assert e.value.code == amr.AMR_ERR_CAPACITY
    assert g.size == len(g.ids()) == len(g.levels())


def test_single_tree_graph_equals_host_driven_and_cluster(amr):
    """One tree past the cluster kernel's limit: graph replays, host-driven
    launches and the cluster kernel (with hand-over) agree bit for bit."""
    import amr_gb300 as A

    rank, n, h = 2, 16, 1
    b = A.seeded_bumps(2, 12, 5, sigma=(0.03, 0.06), amp=(0.5, 2.0), lo=0.05, hi=0.95)
    res = []
    for mode in ("cluster", "graph", "host"):
        t = amr.Tree(rank, n, h, 7, capacity=40000)
        t.refine_uniform(4)
        t.upload_state(A.gaussian_state(t.ids(), rank, n, h, 7, b))
        t.halo_exchange()
        st = t.run(33, 4, (0.8, -0.6), 0.4, "grad", 0.02, 0.004, 2, 6, per_launch=(mode != "cluster"),
                   graph=(mode != "host"))
        if mode == "graph":
            assert st["graph_intervals"] == st["intervals"] and st["persistent_intervals"] == 0
        if mode == "host":
            assert st["graph_intervals"] == 0 and st["persistent_intervals"] == 0
        res.append(({k: st[k] for k in ("sum_dt", "executed_steps", "cell_updates", "remeshes", "intervals")},
                    t.ids(), interior(t.download_state(), rank, n, h)))
    for r in res[1:]:
        assert r[0] == res[0][0]
        np.testing.assert_array_equal(r[1], res[0][1])
        np.testing.assert_array_equal(r[2], res[0][2])


def test_graph_path_with_odd_interval_and_max_criterion(amr, oracle_mod):
    """An odd interval (the state ends in the other buffer) and the max-value
    criterion, graph vs host-driven, FP64 and FP32."""
    o = oracle_mod.OracleTree(2, 16, 1, 6, 4096)
    o.refine_all(3)
    o.init_state([0.3, 0.3, 0.05, 1.0, 0.7, 0.6, 0.04, 1.5])
    o.halo_exchange()
    for dt in (amr.F64, amr.F32):
        res = []
        for graph in (True, False):
            t = amr.Tree(2, 16, 1, 6, capacity=8192, dtype=dt)
            t.refine_uniform(3)
            t.upload_state(o.state())
            st = t.run(23, 3, (1.0, 0.5), 0.4, "max", 0.5, 0.1, 1, 5, per_launch=True, graph=graph)
            res.append(((st["sum_dt"], st["executed_steps"], st["cell_updates"]), t.ids(),
                        t.download_state()))
        assert res[0][0] == res[1][0]
        np.testing.assert_array_equal(res[0][1], res[1][1])
        np.testing.assert_array_equal(interior(res[0][2], 2, 16, 1), interior(res[1][2], 2, 16, 1))
