"""The single-tree configurations at their full stated length, on the device
against the oracle (the C restatement, itself pinned bit-exact to the
reference's own runs of the same configurations, shortened, in
test_oracle_golden.py):

  * config 2: 2D active AMR, 16x16 patches, max level 5, two seeded
    Gaussian bumps + 1e-3 seeded noise, v = (1, 0.5), CFL 0.4, re-mesh every
    10 steps, all 2000 steps;
  * config 3: 3D active AMR, 8^3 patches, max level 4 (the stated depth),
    four seeded Gaussian blobs, v = (1, 0.7, 0.3), re-mesh every 10 steps,
    all 500 steps.

Bars: flags and the tree (Morton ids, neighbour tables) after every re-mesh
bit-exact; the sum of the step sizes exact; the FP64 interior state within
1e-12 relative L2 at every re-mesh and at the end.
"""
import numpy as np
import pytest

from conftest import bumps_of, interior, load_golden, neighbors_linear, rel_l2, vel_of

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-12


@pytest.fixture(scope="module")
def amr():
    import amr_gb300 as A

    A.lib()
    return A


def _tables(tree, rank):
    """Device neighbour records in the oracle comparison layout."""
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


@pytest.mark.parametrize("name,steps,max_level", [("config2_amr_2d", 2000, 5), ("config3_amr_3d", 500, 4)])
def test_full_length_config_against_oracle(amr, oracle_mod, name, steps, max_level):
    O = oracle_mod
    O.set_threads(16)
    _, meta = load_golden(name)
    p = meta["params"]
    rank, n, h, depth = meta["rank"], meta["n"], meta["halo"], meta["depth"]
    vel, cfl, interval = vel_of(meta), float(p["cfl"]), int(p["remesh"])
    rthr, cthr, minl = float(p["rthr"]), float(p["cthr"]), int(p["min_level"])
    o = O.OracleTree(rank, n, h, depth, 20000)
    o.refine_all(int(p["init_levels"]))
    o.init_state(bumps_of(meta), float(p.get("noise", 0.0)), int(p.get("noise_seed", 0)))
    o.halo_exchange()
    t = amr.Tree(rank, n, h, depth, capacity=20000)
    t.refine_uniform(int(p["init_levels"]))
    np.testing.assert_array_equal(t.ids(), o.ids())
    t.upload_state(o.state())
    t.halo_exchange()
    done, sum_t, sum_o, remeshes, changed = 0, 0.0, 0.0, 0, 0
    while done < steps:
        k = min(interval, steps - done)
        t.advance(k, vel, cfl)
        acc_t, ex = t.finish_advance()
        acc_o, ex_o = o.advance(k, vel, cfl)
        assert ex == ex_o == k
        sum_t += acc_t
        sum_o += acc_o
        done += ex
        assert rel_l2(interior(t.download_state(), rank, n, h), interior(o.state(), rank, n, h)) <= STATE_TOL
        fo = o.flags_gradient(rthr, cthr, minl, max_level)
        t.flags_gradient(rthr, cthr, minl, max_level)
        np.testing.assert_array_equal(t.get_flags(), fo)
        before = o.ids()
        assert o.reconstruct(fo) == 0
        o.halo_exchange()
        t.remesh()
        np.testing.assert_array_equal(t.ids(), o.ids())
        for a, b in zip(_tables(t, rank), neighbors_linear(o.ids(), o.neighbors(), rank)):
            np.testing.assert_array_equal(a, b)
        remeshes += 1
        changed += int(len(before) != len(o.ids()) or not np.array_equal(before, o.ids()))
    assert done == steps and remeshes == steps // interval
    assert sum_t == sum_o
    assert changed > 0  # the configuration adapts
    t.halo_exchange()
    err = rel_l2(interior(t.download_state(), rank, n, h), interior(o.state(), rank, n, h))
    assert err <= STATE_TOL, err
