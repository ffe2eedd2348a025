"""SSPRK2 / SSPRK3 steps of advection on the device tree, through the C ABI.

Bars (bit-exact throughout):
  * against the reference's own integrator classes driving the FV residual
    (golden fixtures of the reference, 2D and 3D, with gradient re-meshes):
    flags and trees at every re-mesh, the final state's interior and face
    ghosts, the simulated time;
  * against the oracle on a 2:1 mesh with every neighbour relation, with a
    time limit that cuts the run short (executed steps and time equal).
"""
import numpy as np
import pytest

from conftest import face_mask, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def amr():
    import amr_gb300 as A

    A.lib()
    return A


@pytest.mark.parametrize("name", ["ssprk2_advection_2d", "ssprk3_advection_2d", "ssprk3_advection_3d"])
def test_ssprk_matches_reference_run(amr, name):
    z, meta = load_golden(name)
    p = meta["params"]
    rank, n, h = meta["rank"], meta["n"], meta["halo"]
    t = amr.Tree(rank, n, h, meta["depth"], capacity=40000, dtype=amr.F64)
    t.refine_uniform(int(p["init_levels"]))
    np.testing.assert_array_equal(t.ids(), z["ids_init"])
    t.upload_state(z["state_init"])
    t.halo_exchange()
    vel = [float(x) for x in str(p["vel"]).split(",")]
    steps, interval, order = int(p["steps"]), int(p["remesh"]), int(p["order"])
    done, time, k = 0, 0.0, 0
    while done < steps:
        t.advance_ssprk(min(interval, steps - done), order, vel, float(p["cfl"]))
        acc, ex = t.finish_advance()
        time += acc
        done += ex
        if done % interval == 0:
            t.flags_gradient(float(p["rthr"]), float(p["cthr"]), int(p["min_level"]), int(p["max_level"]))
            np.testing.assert_array_equal(t.get_flags(), z[f"flags_{k}"])
            t.remesh()
            np.testing.assert_array_equal(t.ids(), z[f"ids_{k}"])
            k += 1
    assert k == int(z["remeshes"]) and done == int(z["steps"])
    assert time == float(z["time"])
    t.halo_exchange()
    m = face_mask(rank, n, h)
    np.testing.assert_array_equal(t.download_state()[..., m], z["state_final"][..., m])


@pytest.mark.parametrize("order", [2, 3])
def test_ssprk_matches_oracle_with_time_limit(amr, oracle_mod, order):
    rank, n, h, vel, cfl = 2, 8, 1, (-0.6, 0.9), 0.4
    o = oracle_mod.OracleTree(rank, n, h, 6, 20000)
    t = amr.Tree(rank, n, h, 6, capacity=20000, dtype=amr.F64)
    o.refine_all(1)
    t.refine_uniform(1)
    for k in range(2):
        f = o.flags_random(31, k + 1, 0.4, 0.3, 1, 4)
        assert o.reconstruct(f) == 0
        t.set_flags(f)
        t.remesh()
    np.testing.assert_array_equal(t.ids(), o.ids())
    o.random_state(8)
    o.halo_exchange()
    t.upload_state(o.state())
    dt0 = o.compute_dt(vel, cfl)
    for steps, remaining in ((6, 1.7976931348623157e308), (8, 3.5 * dt0)):
        acc_o, ex_o = o.ssprk_advance(steps, order, vel, cfl, remaining)
        t.advance_ssprk(steps, order, vel, cfl, remaining)
        acc, ex = t.finish_advance()
        assert (acc, ex) == (acc_o, ex_o)
        # the whole padded state: interior and the combined ghosts alike
        m = face_mask(rank, n, h)
        np.testing.assert_array_equal(t.download_state()[..., m], o.state()[..., m])
    assert ex_o == 4  # the limit cut the second advance
