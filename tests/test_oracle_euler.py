"""The oracle's Euler restatement (EulerPhysics<DIM> through amr_solver)
against the reference run from its own headers: the acoustic pulse of the
reference's Euler benchmark on a 1000^rank domain, max-Rho criterion, 2D and
3D.  Bar: trees, flags and every field of every interior and face-ghost cell
bit-exact, simulated time exact."""
import numpy as np
import pytest

from conftest import face_mask, load_golden


def masked(state, rank, n, h):
    """Interior and face-ghost cells of every field (edge and corner ghosts
    are never written by the reference's face halo exchange; its debug build
    fills them with -1000 on buffer swaps)."""
    m = face_mask(rank, n, h)
    return state[..., m]


def euler_reference_loop(O, name):
    z, meta = load_golden(name)
    p = meta["params"]
    rank, n, h, nvar = meta["rank"], meta["n"], meta["halo"], meta["nvar"]
    t = O.OracleTree(rank, n, h, meta["depth"], 40000, nvar=nvar, lengths=meta["lengths"])
    t.refine_all(int(p["init_levels"]))
    np.testing.assert_array_equal(t.ids(), z["ids_init"])
    t.euler_init_pulse(gamma=float(p["gamma"]))
    t.halo_exchange()
    return z, meta, t


@pytest.mark.parametrize("name", ["euler_pulse_2d", "euler_pulse_3d"])
def test_oracle_euler_matches_reference(oracle_mod, name):
    z, meta, t = euler_reference_loop(oracle_mod, name)
    p = meta["params"]
    rank, n, h = meta["rank"], meta["n"], meta["halo"]
    np.testing.assert_array_equal(masked(t.state(), rank, n, h), masked(z["state_init"], rank, n, h))
    gamma, cfl = float(p["gamma"]), float(p["cfl"])
    steps, interval = int(p["steps"]), int(p["remesh"])
    done, time, k = 0, 0.0, 0
    while done < steps:
        acc, ex, _ = t.euler_advance(min(interval, steps - done), gamma, cfl)
        time += acc
        done += ex
        f = t.flags_max(0.53, 0.49, int(p["min_level"]), int(p["max_level"]))
        np.testing.assert_array_equal(f, z[f"flags_{k}"])
        assert t.reconstruct(f) == 0
        t.halo_exchange()
        np.testing.assert_array_equal(t.ids(), z[f"ids_{k}"])
        k += 1
    assert k == int(z["remeshes"])
    assert time == float(z["time"]) and done == int(z["steps"])
    np.testing.assert_array_equal(masked(t.state(), rank, n, h), masked(z["state_final"], rank, n, h))
