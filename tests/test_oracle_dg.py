"""The numpy DG restatement (oracle/dg_oracle.py) against fixtures produced
by running the reference's own DG patch solver: initial state, every step
and the step sizes, bit for bit."""
import numpy as np
import pytest

from oracle import dg_oracle as G
from dg_cases import CASES, EULER_CASES, fixture_tree, load, printer_cases


@pytest.mark.parametrize("name", CASES)
def test_dg_oracle_matches_reference(name):
    z = load(name)
    L = int(z["level"])
    st, dts = z["state"], z["dt"]
    np.testing.assert_array_equal(G.to_leaves(G.initial_state(L), L), st[0])
    outs, mine = G.run(L, len(st) - 1, dt0=float(dts[1]), U=G.from_leaves(st[0], L))
    for k, U in enumerate(outs, start=1):
        np.testing.assert_array_equal(G.to_leaves(U, L), st[k])
    np.testing.assert_array_equal(np.array(mine), dts[1:])


@pytest.mark.parametrize("name", EULER_CASES)
def test_dg_euler_oracle_matches_reference(name):
    """The DG Euler equations (flux, pressure, the patch's running maximum of
    the face speeds, the CFL step from the last stage) from the reference's
    initial state: every step and step size bit for bit.  The initial state
    itself is compared within 4 ulp: the pulse exp(-100 r^2) comes from the
    C library's exp there and numpy's here."""
    z = load(name)
    L = int(z["level"])
    st, dts = z["state"], z["dt"]
    np.testing.assert_allclose(G.to_leaves(G.euler_initial_state(L), L), st[0], rtol=4 * 2.0 ** -52, atol=0)
    outs, mine = G.run(L, len(st) - 1, dt0=float(dts[1]), U=G.from_leaves(st[0], L), equation="euler")
    for k, U in enumerate(outs, start=1):
        np.testing.assert_array_equal(G.to_leaves(U, L), st[k])
    np.testing.assert_array_equal(np.array(mine), dts[1:])
    assert dts[2] < dts[1]  # the wave speeds set the step after the first


def test_dg_tables_match_the_basis():
    """Face kernels reproduce constants (partition of unity) and the
    derivative rows sum to zero (derivative of a constant)."""
    T = G.tables()
    assert abs(T["kern"][0].sum() - 1.0) < 1e-15 and abs(T["kern"][1].sum() - 1.0) < 1e-15
    assert np.all(np.abs(T["D"].sum(axis=0)) < 1e-15)
    np.testing.assert_array_equal(T["mass"], np.full((2, 2), 0.25))


def test_dg_oracle_advects_a_constant_unchanged():
    """A constant field is a steady state of the residual."""
    U = np.ones((8, 8, 2, 2, 4))
    R = G.rhs(U, 1.0 / 8)
    assert np.all(np.abs(R) < 1e-12)


def test_dg_main_loop_fixture_is_consistent():
    """The reference main-loop record: the loop stopped at the first time
    >= end (time grows by the updated step), re-meshed after step 1 and then
    every `amr` steps, and its final leaves are sorted, unique Morton ids of
    levels 1..6 whose cells make up the unit square."""
    z = load("dg_main_loop")
    end, every, steps = float(z["end"]), int(z["amr"]), int(z["steps"])
    assert z["time"] >= end and z["time"] - z["next_dt"] < end
    assert int(z["remeshes"]) == 1 + (steps - 1) // every
    ids = z["ids"]
    assert np.all(ids[1:] > ids[:-1]) and len(ids) <= int(z["leaves_max"])
    levels = (ids & np.uint64(63)).astype(int)
    assert levels.min() >= 1 and levels.max() <= 6
    assert np.sum(4.0 ** -levels) == 1.0
    assert int(z["cells"]) % 16 == 0 and 16 * steps <= int(z["cells"]) <= 16 * int(z["leaves_max"]) * steps
    # the record is the tree at the end of the loop, not the uniform start
    L = int(z["level"])
    assert not (len(ids) == 4 ** L and np.all(levels == L))


@pytest.mark.parametrize("name", sorted(printer_cases()))
def test_dg_printer_oracle_matches_reference(name):
    """The numpy restatement of the reference's DG printer against the files
    the reference's dg_tree_printer_2d wrote for the same trees (uniform
    level 2, and the re-meshed advection and Euler trees over levels 3-6):
    byte for byte (SHA-256 and length)."""
    import hashlib

    c = printer_cases()[name]
    ids, leaves = fixture_tree(c["fixture"], c["dump"])
    b = G.dg_vtk_bytes(ids, leaves)
    assert len(b) == c["bytes"] and hashlib.sha256(b).hexdigest() == c["sha256"]
