"""Pins the C restatement (oracle/) against dumps of the real reference
(tests/golden/, generated by tests/golden/make_golden.py from the reference's
own headers).  Everything here must match bit for bit."""
import numpy as np
import pytest

from conftest import bumps_of, face_mask, interior, load_golden, neighbors_linear, vel_of


def _assert_tables(t, z, k, rank):
    ids = t.ids()
    np.testing.assert_array_equal(ids, z[f"ids_{k}"])
    kind, nbid, quad = neighbors_linear(ids, t.neighbors(), rank)
    np.testing.assert_array_equal(kind, z[f"kind_{k}"])
    np.testing.assert_array_equal(nbid, z[f"nbid_{k}"])
    np.testing.assert_array_equal(quad, z[f"quad_{k}"])


@pytest.mark.parametrize("name", ["config1_uniform_2d", "config2_amr_2d", "config3_amr_3d"])
def test_solver_runs_match_reference(oracle_mod, name):
    z, meta = load_golden(name)
    p = meta["params"]
    rank, n, h = meta["rank"], meta["n"], meta["halo"]
    t = oracle_mod.OracleTree(rank, n, h, meta["depth"])
    t.refine_all(int(p["init_levels"]))
    np.testing.assert_array_equal(t.ids(), z["init_ids"])
    t.init_state(bumps_of(meta), float(p.get("noise", 0.0)), int(p.get("noise_seed", 0)))
    np.testing.assert_array_equal(interior(t.state(), rank, n, h), z["state_init"])
    t.halo_exchange()
    steps, interval = int(p["steps"]), int(p["remesh"])
    vel, cfl = vel_of(meta), float(p["cfl"])
    done, sum_dt, k, mid = 0, 0.0, 0, 0
    while done < steps:
        todo = min(interval, steps - done) if interval > 0 else steps - done
        acc, ex = t.advance(todo, vel, cfl)
        sum_dt += acc
        done += ex
        if interval > 0 and p["crit"] != "none":
            if f"state_mid_{mid}" in z and int(z[f"state_mid_step_{mid}"]) == done:
                np.testing.assert_array_equal(interior(t.state(), rank, n, h), z[f"state_mid_{mid}"])
                mid += 1
            f = t.flags_gradient(float(p["rthr"]), float(p["cthr"]), int(p["min_level"]), int(p["max_level"]))
            np.testing.assert_array_equal(f, z[f"flags_{k}"])
            assert t.reconstruct(f) == 0
            t.halo_exchange()
            _assert_tables(t, z, k, rank)
            k += 1
    assert k == int(z["n_remesh"])
    assert done == int(z["steps"])
    assert sum_dt == float(z["sum_dt"])
    np.testing.assert_array_equal(t.ids(), z["final_ids"])
    np.testing.assert_array_equal(interior(t.state(), rank, n, h), z["state_final"])


@pytest.mark.parametrize(
    "name", ["tree_random_2d_n4", "tree_random_2d_n8", "tree_random_3d_n4", "tree_random_2d_h2"]
)
def test_tree_cycles_match_reference(oracle_mod, name):
    z, meta = load_golden(name)
    p = meta["params"]
    rank, n, h = meta["rank"], meta["n"], meta["halo"]
    seed = int(p["seed"])
    t = oracle_mod.OracleTree(rank, n, h, meta["depth"])
    t.refine_all(int(p["init_levels"]))
    t.random_state(seed * 7919 + 17)
    t.halo_exchange()
    np.testing.assert_array_equal(t.ids(), z["ids_init"])
    m = face_mask(rank, n, h).reshape(-1)
    for k in range(int(z["passes"])):
        f = t.flags_random(seed, k + 1, float(p["p_refine"]), float(p["p_coarsen"]),
                           int(p["min_level"]), int(p["max_level"]))
        np.testing.assert_array_equal(f, z[f"flags_{k}"])
        assert t.reconstruct(f) == 0
        t.halo_exchange()
        _assert_tables(t, z, k, rank)
        if f"state_{k}" in z:
            a = t.state().reshape(t.size, -1)[:, m]
            b = z[f"state_{k}"].reshape(t.size, -1)[:, m]
            np.testing.assert_array_equal(a, b)


def test_morton_roundtrip_and_family(oracle_mod):
    L = oracle_mod.lib()
    import ctypes as C

    rng = np.random.default_rng(0)
    for rank, depth in ((2, 7), (3, 7), (2, 29), (3, 19)):
        for _ in range(200):
            level = int(rng.integers(0, depth + 1))
            cell = 1 << (depth - level)
            c = (rng.integers(0, 1 << level, size=3) * cell).astype(np.uint32)
            c = np.ascontiguousarray(c)
            id_ = L.oracle_encode(rank, depth, c, level)
            out = np.zeros(3, np.uint32)
            lv = C.c_int(0)
            L.oracle_decode(rank, id_, out, C.byref(lv))
            assert lv.value == level
            np.testing.assert_array_equal(out[:rank], c[:rank])
            if level < depth:
                for off in range(2**rank):
                    ch = L.oracle_child_of(rank, depth, id_, off)
                    assert L.oracle_parent_of(rank, depth, ch) == id_
                    assert (ch & 63) == level + 1


def test_known_answer_pulse_moves_with_velocity(oracle_mod):
    """The reference's PulseCenterMovement (tests/advection_equation_amr.t.cpp:50-130):
    root-only tree, 50x50 cells, halo 2, Gaussian exp(-r^2/0.005) at (0.2, 0.2),
    advance to t=0.5; the maximum must sit within one cell of start + v t."""
    t = oracle_mod.OracleTree(2, 50, 2, 7, 16)
    # exp(-r^2/0.005) == exp(-r^2/(2 s^2)) with s^2 = 0.0025
    t.init_state([0.2, 0.2, 0.05, 1.0])
    t.halo_exchange()
    tt, target = 0.0, 0.5
    while tt < target:
        acc, ex = t.advance(1, [1.0, 0.5], 0.4)
        tt += acc
    u = interior(t.state(), 2, 50, 2)[0]
    iy, ix = np.unravel_index(np.argmax(u), u.shape)
    x, y = (ix + 0.5) / 50, (iy + 0.5) / 50
    assert abs(x - 0.7) <= 1 / 50 and abs(y - 0.45) <= 1 / 50
