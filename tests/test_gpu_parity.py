"""CUDA path vs the reference (golden dumps) and the oracle, through the C ABI.

Bars (stated per test):
  * Morton ids, neighbour tables, refine/coarsen flags, tree after every
    re-mesh: bit-exact.
  * Halo ghosts, prolongation, restriction on identical inputs: bit-exact.
  * FP64 cell states after many steps: relative L2 <= 1e-12 (the fused
    kernel evaluates the upwind form of the Rusanov flux with FMA).
  * Sum of time steps: exact.
"""
import numpy as np
import pytest

from conftest import bumps_of, face_mask, interior, load_golden, rel_l2, vel_of

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-12


@pytest.fixture(scope="module")
def amr():
    import amr_gb300 as A

    A.lib()
    return A


def _pad(inner, rank, n, h):
    P1 = n + 2 * h
    out = np.zeros((inner.shape[0],) + (P1,) * rank)
    out[(slice(None),) + (slice(h, n + h),) * rank] = inner
    return out


def _tables(tree, rank):
    nb = tree.neighbors()
    kind = nb["relation"].astype(np.int8)
    nbid = np.full(nb["finer_ids"].shape, -1, np.int32)
    same = (kind == 1) | (kind == 3)
    nbid[..., 0][same] = nb["neighbor"][same]
    nf = 2 ** (rank - 1)
    fin = kind == 2
    nbid[..., :nf][fin] = nb["finer_ids"][..., :nf][fin]
    quad = nb["quadrant"].astype(np.int8)
    quad[kind != 3] = 0
    return kind, nbid, quad


def _assert_tables(tree, z, k, rank):
    np.testing.assert_array_equal(tree.ids(), z[f"ids_{k}"])
    kind, nbid, quad = _tables(tree, rank)
    np.testing.assert_array_equal(kind, z[f"kind_{k}"])
    np.testing.assert_array_equal(nbid, z[f"nbid_{k}"])
    np.testing.assert_array_equal(quad, z[f"quad_{k}"])


@pytest.mark.parametrize("name", ["config1_uniform_2d", "config2_amr_2d", "config3_amr_3d"])
def test_solver_run_matches_reference(amr, name):
    z, meta = load_golden(name)
    p = meta["params"]
    rank, n, h = meta["rank"], meta["n"], meta["halo"]
    t = amr.Tree(rank, n, h, meta["depth"], capacity=20000)
    t.refine_uniform(int(p["init_levels"]))
    np.testing.assert_array_equal(t.ids(), z["init_ids"])
    t.upload_state(_pad(z["state_init"], rank, n, h))
    t.halo_exchange()
    steps, interval = int(p["steps"]), int(p["remesh"])
    vel, cfl = vel_of(meta), float(p["cfl"])
    done, sum_dt, k, mid = 0, 0.0, 0, 0
    while done < steps:
        todo = min(interval, steps - done) if interval > 0 else steps - done
        t.advance(todo, vel, cfl)
        acc, ex = t.finish_advance()
        sum_dt += acc
        done += ex
        if interval > 0 and p["crit"] != "none":
            if f"state_mid_{mid}" in z and int(z[f"state_mid_step_{mid}"]) == done:
                got = interior(t.download_state(), rank, n, h)
                assert rel_l2(got, z[f"state_mid_{mid}"]) <= STATE_TOL
                mid += 1
            t.flags_gradient(float(p["rthr"]), float(p["cthr"]), int(p["min_level"]), int(p["max_level"]))
            np.testing.assert_array_equal(t.get_flags(), z[f"flags_{k}"])
            t.remesh()
            _assert_tables(t, z, k, rank)
            k += 1
    assert k == int(z["n_remesh"])
    assert done == int(z["steps"])
    assert sum_dt == float(z["sum_dt"])
    np.testing.assert_array_equal(t.ids(), z["final_ids"])
    err = rel_l2(interior(t.download_state(), rank, n, h), z["state_final"])
    assert err <= STATE_TOL, err


@pytest.mark.parametrize(
    "name", ["tree_random_2d_n4", "tree_random_2d_n8", "tree_random_3d_n4", "tree_random_2d_h2"]
)
def test_tree_cycle_matches_reference(amr, name):
    z, meta = load_golden(name)
    p = meta["params"]
    rank, n, h = meta["rank"], meta["n"], meta["halo"]
    t = amr.Tree(rank, n, h, meta["depth"], capacity=20000)
    t.refine_uniform(int(p["init_levels"]))
    np.testing.assert_array_equal(t.ids(), z["ids_init"])
    t.upload_state(z["state_init"])
    m = face_mask(rank, n, h).reshape(-1)
    for k in range(int(z["passes"])):
        t.set_flags(z[f"flags_{k}"])
        t.remesh()
        t.halo_exchange()
        _assert_tables(t, z, k, rank)
        if f"state_{k}" in z:
            a = t.download_state().reshape(t.size, -1)[:, m]
            b = z[f"state_{k}"].reshape(t.size, -1)[:, m]
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("rank,n,h,levels,maxl,seed", [(2, 8, 1, 2, 6, 21), (3, 4, 1, 1, 4, 22), (2, 6, 2, 1, 5, 23)])
def test_random_cycles_against_oracle(amr, oracle_mod, rank, n, h, levels, maxl, seed):
    """Longer random refine/coarsen sequences than the fixtures hold, checked
    against the C restatement on the same inputs."""
    o = oracle_mod.OracleTree(rank, n, h, 7, 40000)
    o.refine_all(levels)
    o.random_state(seed)
    o.halo_exchange()
    t = amr.Tree(rank, n, h, 7, capacity=40000)
    t.refine_uniform(levels)
    t.upload_state(o.state())
    m = face_mask(rank, n, h).reshape(-1)
    for k in range(12):
        f = o.flags_random(seed, k + 1, 0.15, 0.6, 1, maxl)
        assert o.reconstruct(f) == 0
        o.halo_exchange()
        t.set_flags(f)
        t.remesh()
        t.halo_exchange()
        np.testing.assert_array_equal(t.ids(), o.ids())
        a = t.download_state().reshape(t.size, -1)[:, m]
        b = o.state().reshape(o.size, -1)[:, m]
        np.testing.assert_array_equal(a, b)


def test_known_answer_pulse_with_amr(amr, oracle_mod):
    """The reference's PulseCenterMovementAMR (tests/advection_equation_amr.t.cpp:132-232),
    50x50 patches with halo 2: max-value criterion (refine > 0.1 below level 5,
    coarsen < 0.05 above level 1) re-meshing every step, advance to t = 0.5;
    the maximum must sit within one cell of start + v t."""
    rank, n, h = 2, 50, 2
    o = oracle_mod.OracleTree(rank, n, h, 7, 64)
    o.init_state([0.2, 0.2, 0.05, 1.0])
    o.halo_exchange()
    t = amr.Tree(rank, n, h, 7, capacity=4096)
    t.upload_state(o.state())
    tt = 0.0
    while tt < 0.5:
        t.advance(1, [1.0, 0.5], 0.4)
        acc, _ = t.finish_advance()
        t.flags_max(0.1, 0.05, 1, 5)
        t.remesh()
        tt += acc
    t.halo_exchange()
    u = interior(t.download_state(), rank, n, h)
    ids, best = t.ids(), np.unravel_index(np.argmax(u), u.shape)
    p, iy, ix = best
    level = int(ids[p] & 63)
    m = int(ids[p] >> 6)
    x0 = sum(((m >> (2 * b)) & 1) << b for b in range(7)) / 2**7
    y0 = sum(((m >> (2 * b + 1)) & 1) << b for b in range(7)) / 2**7
    dx = 1.0 / (n * 2**level)
    x, y = x0 + (ix + 0.5) * dx, y0 + (iy + 0.5) * dx
    finest = 1.0 / (n * 2 ** int(t.levels().max()))
    assert abs(x - 0.7) <= max(dx, finest) and abs(y - 0.45) <= max(dx, finest)


def test_noop_remesh_and_capacity(amr):
    t = amr.Tree(2, 8, 1, 7, capacity=20)
    t.refine_uniform(1)
    ids = t.ids()
    t.set_flags(np.zeros(4, np.int8))
    assert t.remesh() is False
    np.testing.assert_array_equal(t.ids(), ids)
    t.set_flags(np.ones(4, np.int8))  # 16 leaves fit
    assert t.remesh() is True
    t.set_flags(np.ones(16, np.int8))  # 64 > 20
    with pytest.raises(amr.AmrError) as e:
        t.remesh()
    assert e.value.code == amr.AMR_ERR_CAPACITY
    assert t.size == 16  # tree left unchanged


def test_depth_cap_blocks_refinement(amr):
    t = amr.Tree(2, 4, 1, depth=2, capacity=100)
    t.refine_uniform(2)
    assert t.size == 16
    t.set_flags(np.ones(16, np.int8))  # level == depth: not eligible
    assert t.remesh() is False


def test_invalid_arguments_are_rejected(amr):
    for bad in (dict(rank=4, n=8), dict(rank=2, n=7), dict(rank=2, n=2, halo=2), dict(rank=3, n=8, depth=20)):
        kw = dict(halo=1, depth=7)
        kw.update(bad)
        with pytest.raises(amr.AmrError) as e:
            amr.Tree(capacity=16, **kw)
        assert e.value.code == amr.AMR_ERR_INVALID
    t = amr.Tree(2, 8, 1, 7, capacity=16)
    with pytest.raises(amr.AmrError):
        t.set_flags(np.zeros(3, np.int8))


def test_fp32_form_tracks_fp64(amr):
    """FP32 state/flux with FP64 dt and restriction: same tree, L2 error vs
    the FP64 path below 1e-5 on the shortened config-2 run."""
    z, meta = load_golden("config2_amr_2d")
    p = meta["params"]
    res = {}
    for dt in (amr.F64, amr.F32):
        t = amr.Tree(2, 16, 1, 7, capacity=20000, dtype=dt)
        t.refine_uniform(2)
        t.upload_state(_pad(z["state_init"], 2, 16, 1))
        t.halo_exchange()
        for _ in range(3):
            t.advance(10, vel_of(meta), 0.4)
            t.finish_advance()
            t.flags_gradient(0.05, 0.01, 1, 5)
            t.remesh()
        res[dt] = (t.ids(), interior(t.download_state(), 2, 16, 1).astype(np.float64))
    np.testing.assert_array_equal(res[amr.F64][0], res[amr.F32][0])
    assert rel_l2(res[amr.F32][1], res[amr.F64][1]) <= 1e-5


def _host_loop(amr, t, steps, interval, vel, cfl, crit, rthr, cthr, minl, maxl):
    done, sum_dt, cells = 0, 0.0, 0
    while done < steps:
        k = min(interval, steps - done)
        P = t.size
        t.advance(k, vel, cfl)
        acc, ex = t.finish_advance()
        done += ex
        sum_dt += acc
        cells += ex * P * t.n ** t.rank
        if crit == "grad":
            t.flags_gradient(rthr, cthr, minl, maxl)
        else:
            t.flags_max(rthr, cthr, minl, maxl)
        t.remesh()
        if ex == 0:
            break
    return sum_dt, done, cells


@pytest.mark.parametrize("name", ["config2_amr_2d", "config3_amr_3d"])
def test_persistent_run_matches_host_loop_and_reference(amr, name):
    """amr_tree_run (one cluster kernel per run) == the host-driven loop of
    advance/flags/remesh, bit for bit, and == the reference fixtures."""
    z, meta = load_golden(name)
    p = meta["params"]
    rank, n, h = meta["rank"], meta["n"], meta["halo"]
    args = (int(p["steps"]), int(p["remesh"]), vel_of(meta), float(p["cfl"]))
    crit = (float(p["rthr"]), float(p["cthr"]), int(p["min_level"]), int(p["max_level"]))
    res = []
    for mode in ("run", "host"):
        t = amr.Tree(rank, n, h, meta["depth"], capacity=20000)
        t.refine_uniform(int(p["init_levels"]))
        t.upload_state(_pad(z["state_init"], rank, n, h))
        t.halo_exchange()
        if mode == "run":
            st = t.run(*args, criterion="grad", rthr=crit[0], cthr=crit[1], min_level=crit[2], max_level=crit[3])
            assert st["persistent_intervals"] == st["intervals"] > 0
            out = (st["sum_dt"], st["executed_steps"], st["cell_updates"])
        else:
            out = _host_loop(amr, t, *args, "grad", *crit)
        res.append((out, t.ids(), interior(t.download_state(), rank, n, h)))
    (a, ids_a, s_a), (b, ids_b, s_b) = res
    assert a == b
    np.testing.assert_array_equal(ids_a, ids_b)
    np.testing.assert_array_equal(s_a, s_b)
    assert a[0] == float(z["sum_dt"])
    np.testing.assert_array_equal(ids_a, z["final_ids"])
    assert rel_l2(s_a, z["state_final"]) <= STATE_TOL


def test_persistent_run_hands_over_to_per_launch_kernels(amr):
    """A tree that grows past the cluster kernel's leaf limit continues with
    per-launch kernels; the result equals the host-driven loop."""
    import amr_gb300 as A

    rank, n, h = 2, 8, 1
    b = A.seeded_bumps(2, 40, 11, sigma=(0.03, 0.05), amp=(1.0, 2.0), lo=0.05, hi=0.95)
    res = []
    for mode in ("run", "host"):
        t = amr.Tree(rank, n, h, 7, capacity=40000)
        t.refine_uniform(5)  # 1024 leaves: the cluster kernel's limit
        t.upload_state(A.gaussian_state(t.ids(), rank, n, h, 7, b))
        t.halo_exchange()
        if mode == "run":
            st = t.run(20, 5, (1.0, 0.5), 0.4, "grad", 0.01, 0.002, 1, 6)
            out = (st["sum_dt"], st["executed_steps"], st["cell_updates"])
            assert st["leaves_max"] > 1024 and 0 < st["persistent_intervals"] < st["intervals"]
        else:
            out = _host_loop(amr, t, 20, 5, (1.0, 0.5), 0.4, "grad", 0.01, 0.002, 1, 6)
        res.append((out, t.ids(), interior(t.download_state(), rank, n, h)))
    assert res[0][0] == res[1][0]
    np.testing.assert_array_equal(res[0][1], res[1][1])
    np.testing.assert_array_equal(res[0][2], res[1][2])


def test_persistent_run_max_criterion_and_fp32(amr, oracle_mod):
    """Max-value criterion and FP32 state through the cluster kernel equal the
    host-driven loop on the same inputs."""
    o = oracle_mod.OracleTree(2, 10, 2, 7, 64)
    o.init_state([0.2, 0.2, 0.05, 1.0])
    o.halo_exchange()
    for dt in (amr.F64, amr.F32):
        res = []
        for mode in ("run", "host"):
            t = amr.Tree(2, 10, 2, 7, capacity=4096, dtype=dt)
            t.upload_state(o.state())
            if mode == "run":
                st = t.run(40, 1, (1.0, 0.5), 0.4, "max", 0.1, 0.05, 1, 5)
                out = (st["sum_dt"], st["executed_steps"])
            else:
                out = _host_loop(amr, t, 40, 1, (1.0, 0.5), 0.4, "max", 0.1, 0.05, 1, 5)[:2]
            res.append((out, t.ids(), interior(t.download_state(), 2, 10, 2)))
        assert res[0][0] == res[1][0]
        np.testing.assert_array_equal(res[0][1], res[1][1])
        np.testing.assert_array_equal(res[0][2], res[1][2])


@pytest.mark.parametrize("n,h", [(16, 1), (8, 1), (6, 2)])
@pytest.mark.parametrize("vel", [(1.0, 0.5), (-1.0, 0.5), (0.7, -0.3), (-0.6, -0.9), (0.0, 1.0), (-0.4, 0.0)])
def test_update_all_velocity_signs_against_oracle(amr, oracle_mod, n, h, vel):
    """The fused update (the compile-time-sized 2D kernel for 16^2 and 8^2
    patches, the generic kernel otherwise) on an irregular 2:1 tree, for every
    upwind direction, against the reference's flux on the same input."""
    rank, seed = 2, 31
    o = oracle_mod.OracleTree(rank, n, h, 7, 20000)
    o.refine_all(2)
    for k in range(3):
        assert o.reconstruct(o.flags_random(seed, k + 1, 0.3, 0.5, 1, 5)) == 0
    o.random_state(seed)
    o.halo_exchange()
    t = amr.Tree(rank, n, h, 7, capacity=20000)
    t.refine_uniform(2)
    # the same tree on the GPU from the same flag sequence
    o2 = oracle_mod.OracleTree(rank, n, h, 7, 20000)
    o2.refine_all(2)
    for k in range(3):
        f = o2.flags_random(seed, k + 1, 0.3, 0.5, 1, 5)
        assert o2.reconstruct(f) == 0
        t.set_flags(f)
        t.remesh()
    np.testing.assert_array_equal(t.ids(), o.ids())
    t.upload_state(o.state())
    acc_o, ex_o = o.advance(5, vel, 0.4)
    t.advance(5, vel, 0.4)
    acc_t, ex_t = t.finish_advance()
    assert (acc_t, ex_t) == (acc_o, ex_o)
    a = interior(t.download_state(), rank, n, h)
    b = interior(o.state(), rank, n, h)
    assert rel_l2(a, b) <= STATE_TOL


def test_bounded_wait_reports_timeout_and_context_survives(amr):
    """A bulk-copy wait that never completes gives up after its poll limit,
    records AMR_ERR_TIMEOUT for the host, and leaves the context usable (a
    follow-up kernel and a full tree run afterwards)."""
    import ctypes as C

    obs = C.c_int32(-1)
    amr.check(amr.lib().amr_selftest_wait_timeout(1 << 12, C.byref(obs)))
    assert obs.value == 7  # AMR_ERR_TIMEOUT
    t = amr.Tree(2, 16, 1, 5, capacity=1024)
    t.refine_uniform(2)
    t.upload_state(np.random.default_rng(0).random((t.size, 18, 18)))
    st = t.run(20, 10, (1.0, 0.5), 0.4, "grad", 0.05, 0.01, 1, 3)
    assert st["executed_steps"] == 20


def test_reserve_keeps_the_tree_and_runs_continue(amr):
    """amr_tree_reserve grows (and shrinks) the capacity in place: leaves,
    state and tables survive, and a run continued after it equals the run
    without it, on both drivers (the interval graph is re-captured)."""
    import amr_gb300 as A

    b = A.seeded_bumps(2, 6, 4, sigma=(0.03, 0.06), amp=(0.5, 2.0), lo=0.05, hi=0.95)
    res = []
    for grow in (False, True):
        t = amr.Tree(2, 16, 1, 7, capacity=8000)
        t.refine_uniform(4)
        t.upload_state(A.gaussian_state(t.ids(), 2, 16, 1, 7, b))
        t.run(12, 4, (0.8, 0.6), 0.4, "grad", 0.02, 0.004, 2, 6, per_launch=True)
        if grow:
            ids, nb, st = t.ids(), t.neighbors(), t.download_state()
            t.reserve(20000)
            assert t.capacity == 20000
            np.testing.assert_array_equal(t.ids(), ids)
            np.testing.assert_array_equal(t.neighbors(), nb)
            np.testing.assert_array_equal(t.download_state(), st)
        t.run(12, 4, (0.8, 0.6), 0.4, "grad", 0.02, 0.004, 2, 6, per_launch=True)
        if grow:
            t.reserve(t.size)  # shrink to fit
            assert t.capacity == t.size
        res.append((t.ids(), interior(t.download_state(), 2, 16, 1)))
    np.testing.assert_array_equal(res[0][0], res[1][0])
    np.testing.assert_array_equal(res[0][1], res[1][1])
    with pytest.raises(amr.AmrError):
        t.reserve(t.size - 1)


@pytest.mark.parametrize("name", ["config2_amr_2d", "config3_amr_3d"])
def test_persistent_run_cluster_sizes_agree(amr, name):
    """The cluster kernel's work split (thread-block clusters of 16, 8, 4 or
    2 CTAs) changes no result: the same leaves and states, bit for bit."""
    z, meta = load_golden(name)
    p = meta["params"]
    rank, n, h = meta["rank"], meta["n"], meta["halo"]
    res = []
    for cluster in (16, 8, 4, 2):
        t = amr.Tree(rank, n, h, meta["depth"], capacity=20000)
        t.refine_uniform(int(p["init_levels"]))
        t.upload_state(_pad(z["state_init"], rank, n, h))
        t.halo_exchange()
        st = t.run(int(p["steps"]), int(p["remesh"]), vel_of(meta), float(p["cfl"]), criterion="grad",
                   rthr=float(p["rthr"]), cthr=float(p["cthr"]), min_level=int(p["min_level"]),
                   max_level=int(p["max_level"]), cluster=cluster)
        assert st["persistent_intervals"] == st["intervals"] > 0
        res.append((st["sum_dt"], t.ids(), interior(t.download_state(), rank, n, h)))
    for sum_dt, ids, s in res[1:]:
        assert sum_dt == res[0][0]
        np.testing.assert_array_equal(ids, res[0][1])
        np.testing.assert_array_equal(s, res[0][2])
