"""The oracle's SSPRK2 / SSPRK3 restatement against the reference's own
integrator classes (include/dg_helpers/time_integration/time.hpp) driving
the FV advection residual on the reference tree (golden fixtures of
oracle/ref_driver mode=ssprk): flags and trees at every re-mesh, every
interior and face-ghost cell of the final state, and the simulated time,
bit-exact.  As in the reference, a step's stages combine whole padded
patches and the criterion after a step sees the combined ghost cells (no
halo exchange between the last stage and the re-mesh)."""
import numpy as np
import pytest

from conftest import bumps_of, face_mask, load_golden


def ssprk_reference_loop(O, name):
    z, meta = load_golden(name)
    p = meta["params"]
    rank, n, h = meta["rank"], meta["n"], meta["halo"]
    t = O.OracleTree(rank, n, h, meta["depth"], 40000)
    t.refine_all(int(p["init_levels"]))
    np.testing.assert_array_equal(t.ids(), z["ids_init"])
    t.set_state(z["state_init"])
    t.halo_exchange()
    return z, meta, t


@pytest.mark.parametrize("name", ["ssprk2_advection_2d", "ssprk3_advection_2d", "ssprk3_advection_3d"])
def test_oracle_ssprk_matches_reference(oracle_mod, name):
    z, meta, t = ssprk_reference_loop(oracle_mod, name)
    p = meta["params"]
    rank, n, h = meta["rank"], meta["n"], meta["halo"]
    vel = [float(x) for x in str(p["vel"]).split(",")]
    steps, interval, order = int(p["steps"]), int(p["remesh"]), int(p["order"])
    done, time, k = 0, 0.0, 0
    while done < steps:
        acc, ex = t.ssprk_advance(min(interval, steps - done), order, vel, float(p["cfl"]))
        time += acc
        done += ex
        if done % interval == 0:
            f = t.flags_gradient(float(p["rthr"]), float(p["cthr"]), int(p["min_level"]), int(p["max_level"]))
            np.testing.assert_array_equal(f, z[f"flags_{k}"])
            assert t.reconstruct(f) == 0
            t.halo_exchange()
            np.testing.assert_array_equal(t.ids(), z[f"ids_{k}"])
            k += 1
    assert k == int(z["remeshes"]) and done == int(z["steps"])
    assert time == float(z["time"])
    t.halo_exchange()
    m = face_mask(rank, n, h)
    np.testing.assert_array_equal(t.state()[..., m], z["state_final"][..., m])
