"""Compressible Euler (EulerPhysics<DIM> through amr_solver) on the device
tree, through the C ABI.

Bars:
  * against the reference's own run (golden fixtures made by the reference
    compiled from its headers; acoustic pulse, max-Rho criterion, 2D and
    3D): flags and trees at every re-mesh, every field of every interior and
    face-ghost cell, and the simulated time, bit-exact;
  * against the oracle on 2:1 meshes with every neighbour relation, seeded
    states with flow in every direction, and a time limit that clamps the
    last step: bit-exact on the same cells, step counts and time exact;
  * amr_tree_euler_run (the benchmark loop with an end time) against the
    oracle's loop: trees, state and time bit-exact;
  * the multi-field VTK file byte-identical to the oracle's writer.
"""
import numpy as np
import pytest

from conftest import face_mask, load_golden

pytestmark = pytest.mark.gpu

DBL_MAX = 1.7976931348623157e308


@pytest.fixture(scope="module")
def amr():
    import amr_gb300 as A

    A.lib()
    return A


def fields_first(state):
    """Oracle layout (size, nvar, ...) -> tree layout (nvar, size, ...)."""
    return np.ascontiguousarray(np.moveaxis(state, 1, 0))


def masked_tree(state, rank, n, h):
    """(nvar, size, ...) -> the interior and face-ghost cells."""
    return state[..., face_mask(rank, n, h)]


def masked_oracle(state, rank, n, h):
    return fields_first(state)[..., face_mask(rank, n, h)]


def _tree(amr, meta, capacity=40000):
    return amr.Tree(meta["rank"], meta["n"], meta["halo"], meta["depth"], capacity=capacity, dtype=amr.F64,
                    lengths=meta["lengths"], fields=meta["nvar"])


@pytest.mark.parametrize("name", ["euler_pulse_2d", "euler_pulse_3d"])
def test_euler_matches_reference_run(amr, name):
    z, meta = load_golden(name)
    p = meta["params"]
    rank, n, h = meta["rank"], meta["n"], meta["halo"]
    t = _tree(amr, meta)
    t.refine_uniform(int(p["init_levels"]))
    np.testing.assert_array_equal(t.ids(), z["ids_init"])
    t.upload_state(fields_first(z["state_init"]))
    t.halo_exchange()
    gamma, cfl = float(p["gamma"]), float(p["cfl"])
    steps, interval = int(p["steps"]), int(p["remesh"])
    done, time, k = 0, 0.0, 0
    while done < steps:
        t.euler_advance(min(interval, steps - done), gamma, cfl)
        t.flags_max(0.53, 0.49, int(p["min_level"]), int(p["max_level"]))
        np.testing.assert_array_equal(t.get_flags(), z[f"flags_{k}"])
        t.remesh()
        np.testing.assert_array_equal(t.ids(), z[f"ids_{k}"])
        acc, ex = t.finish_advance()
        time += acc
        done += ex
        k += 1
    assert k == int(z["remeshes"])
    assert time == float(z["time"]) and done == int(z["steps"])
    t.halo_exchange()
    np.testing.assert_array_equal(masked_tree(t.download_state(), rank, n, h),
                                  masked_oracle(z["state_final"], rank, n, h))


def _flow_state(o, rng, gamma):
    """Positive density and pressure with velocities of both signs along
    every axis: the pulse plus seeded momentum (pressure kept)."""
    o.euler_init_pulse(gamma=gamma, centre=(370.0, 610.0, 450.0))
    s = o.state()
    rank = o.rank
    isl = (slice(o.halo, o.n + o.halo),) * rank
    rho = s[(slice(None), 0) + isl]
    kin = np.zeros_like(rho)
    for d in range(rank):
        m = rng.uniform(-0.6, 0.6, rho.shape) * rho
        s[(slice(None), 1 + d) + isl] = m
        kin += m * m
    s[(slice(None), rank + 1) + isl] += 0.5 * kin / rho
    o.set_state(s)
    o.halo_exchange()


MESHES = [(2, 8, 1, 11), (2, 16, 1, 4), (2, 6, 2, 9), (3, 4, 1, 2)]


@pytest.mark.parametrize("rank,n,h,seed", MESHES)
def test_euler_matches_oracle_on_irregular_meshes(amr, oracle_mod, rank, n, h, seed):
    gamma, cfl, L = 1.4, 0.3, (1000.0, 1000.0, 1000.0)
    nvar = rank + 2
    o = oracle_mod.OracleTree(rank, n, h, 6, 20000, nvar=nvar, lengths=L[:rank])
    t = amr.Tree(rank, n, h, 6, capacity=20000, dtype=amr.F64, lengths=L, fields=nvar)
    o.refine_all(1)
    t.refine_uniform(1)
    for k in range(2):
        f = o.flags_random(seed, k + 1, 0.4, 0.3, 1, 4 if rank == 2 else 3)
        assert o.reconstruct(f) == 0
        t.set_flags(f)
        t.remesh()
    np.testing.assert_array_equal(t.ids(), o.ids())
    _flow_state(o, np.random.default_rng(seed), gamma)
    t.upload_state(fields_first(o.state()))
    # unclamped steps, then a time limit that cuts the run short
    dt0 = o.euler_dt(gamma, cfl)
    for steps, remaining in ((7, DBL_MAX), (9, 2.5 * dt0)):
        acc_o, ex_o, _ = o.euler_advance(steps, gamma, cfl, remaining)
        t.euler_advance(steps, gamma, cfl, remaining)
        acc, ex = t.finish_advance()
        assert (acc, ex) == (acc_o, ex_o)
        np.testing.assert_array_equal(masked_tree(t.download_state(), rank, n, h),
                                      masked_oracle(o.state(), rank, n, h))
    assert 2 <= ex_o < 9  # the time limit ended the second advance


def test_euler_run_matches_oracle_loop(amr, oracle_mod):
    """The benchmark loop with an end time: advance `interval` steps with
    the time left, max-Rho flags, re-mesh, until the end time."""
    rank, n, h, depth = 2, 8, 1, 6
    gamma, cfl, interval, end = 1.4, 0.3, 5, 9.0
    rthr, cthr, minl, maxl = 0.53, 0.49, 1, 4
    o = oracle_mod.OracleTree(rank, n, h, depth, 20000, nvar=4, lengths=(1000.0, 1000.0))
    o.refine_all(2)
    o.euler_init_pulse(gamma=gamma)
    o.halo_exchange()
    t = amr.Tree(rank, n, h, depth, capacity=20000, dtype=amr.F64, lengths=(1000.0, 1000.0), fields=4)
    t.refine_uniform(2)
    t.upload_state(fields_first(o.state()))
    st = t.euler_run(10 ** 6, interval, gamma, cfl, end, rthr, cthr, minl, maxl)
    time, done, remeshes, cells = 0.0, 0, 0, 0
    while time < end:
        leaves = o.size
        acc, ex, _ = o.euler_advance(interval, gamma, cfl, end - time)
        f = o.flags_max(rthr, cthr, minl, maxl)
        assert o.reconstruct(f) == 0
        o.halo_exchange()
        time += acc
        done += ex
        remeshes += 1
        cells += ex * leaves * n * n
        if ex == 0:
            break
    assert time >= end
    assert st["sum_dt"] == time and st["executed_steps"] == done and st["remeshes"] == remeshes
    assert st["cell_updates"] == cells
    np.testing.assert_array_equal(t.ids(), o.ids())
    np.testing.assert_array_equal(masked_tree(t.download_state(), rank, n, h), masked_oracle(o.state(), rank, n, h))


def test_euler_vtk_matches_oracle(amr, oracle_mod, tmp_path):
    rank, n, h = 2, 8, 1
    o = oracle_mod.OracleTree(rank, n, h, 5, 4096, nvar=4, lengths=(1000.0, 1000.0))
    o.refine_all(2)
    o.euler_init_pulse()
    o.halo_exchange()
    t = amr.Tree(rank, n, h, 5, capacity=4096, dtype=amr.F64, lengths=(1000.0, 1000.0), fields=4)
    t.refine_uniform(2)
    t.upload_state(fields_first(o.state()))
    t.euler_advance(4, 1.4, 0.3)
    o.euler_advance(4, 1.4, 0.3)
    names = "Rho,Rhou,Rhov,E4"
    t.write_vtk(tmp_path / "gpu.vtk", names)
    o.write_vtk(str(tmp_path / "cpu.vtk"), names)
    assert (tmp_path / "gpu.vtk").read_bytes() == (tmp_path / "cpu.vtk").read_bytes()


def test_euler_reserve_and_field_guards(amr, oracle_mod):
    rank, n, h = 2, 8, 1
    o = oracle_mod.OracleTree(rank, n, h, 5, 4096, nvar=4, lengths=(1000.0, 1000.0))
    o.refine_all(2)
    o.euler_init_pulse()
    o.halo_exchange()
    t = amr.Tree(rank, n, h, 5, capacity=64, dtype=amr.F64, lengths=(1000.0, 1000.0), fields=4)
    t.refine_uniform(2)
    t.upload_state(fields_first(o.state()))
    t.euler_advance(3, 1.4, 0.3)
    t.reserve(500)  # every field moves to the new buffers
    t.euler_advance(3, 1.4, 0.3)
    o.euler_advance(6, 1.4, 0.3)
    np.testing.assert_array_equal(masked_tree(t.download_state(), rank, n, h), masked_oracle(o.state(), rank, n, h))
    with pytest.raises(amr.AmrError) as e:
        t.advance(1, (1.0, 0.5), 0.4)  # the advection update takes one field
    assert e.value.code == amr.AMR_ERR_INVALID
    one = amr.Tree(rank, n, h, 5, capacity=64, dtype=amr.F64)
    with pytest.raises(amr.AmrError) as e:
        one.euler_advance(1, 1.4, 0.3)
    assert e.value.code == amr.AMR_ERR_INVALID
