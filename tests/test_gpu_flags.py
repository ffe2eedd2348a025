"""Gradient flags at the decision boundary, through the C ABI, against the
oracle.  The thresholds are set to gradient values that occur in the state,
so cells sit exactly on (and next to) the refine and coarsen boundaries and
the kernels' FP32 pre-filter must hand them to the exact FP64 evaluation.
Bar: flags bit-exact, for FP64 and FP32 state, with ghosts from the buffer
and ghosts evaluated on the fly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def amr():
    import amr_gb300 as A

    A.lib()
    return A


def _gradients(state, n, h):
    """|grad u| * h of every interior cell (the oracle's arithmetic)."""
    u = state
    c = slice(h, n + h)
    gx = 0.5 * (u[:, c, h + 1:n + h + 1] - u[:, c, h - 1:n + h - 1])
    gy = 0.5 * (u[:, h + 1:n + h + 1, c] - u[:, h - 1:n + h - 1, c])
    return np.sqrt((0.0 + gx * gx) + gy * gy)


@pytest.mark.parametrize("n", [16, 8, 6])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("ghosts", ["buffer", "on_the_fly"])
def test_gradient_flags_on_the_threshold(amr, oracle_mod, n, dtype, ghosts):
    h, seed = 1, 13
    o = oracle_mod.OracleTree(2, n, h, 6, 20000)
    o.refine_all(2)
    t = amr.Tree(2, n, h, 6, capacity=20000, dtype=amr.F64 if dtype == "f64" else amr.F32)
    t.refine_uniform(2)
    for k in range(2):
        f = o.flags_random(seed, k + 1, 0.3, 0.4, 1, 4)
        assert o.reconstruct(f) == 0
        t.set_flags(f)
        t.remesh()
    np.testing.assert_array_equal(t.ids(), o.ids())
    o.random_state(seed)
    if dtype == "f32":
        o.set_state(o.state().astype(np.float32).astype(np.float64))
    o.halo_exchange()
    st = o.state()
    v = np.sort(_gradients(st, n, h).ravel())
    for q_r, q_c in [(0.7, 0.2), (0.5, 0.5), (0.95, 0.05)]:
        rthr = float(v[int(q_r * (v.size - 1))])
        cthr = float(v[int(q_c * (v.size - 1))])
        fo = o.flags_gradient(rthr, cthr, 1, 4)
        if ghosts == "buffer":
            t.upload_state(st)  # the exchanged ghosts, as the caller's
        else:
            z = st.copy()
            z[:, 0, :] = z[:, -1, :] = 0.0
            z[:, :, 0] = z[:, :, -1] = 0.0
            t.upload_state(z)
            t.advance(0, (1.0, 0.5), 0.4)  # no step; the buffer's ghosts are stale now
        t.flags_gradient(rthr, cthr, 1, 4)
        np.testing.assert_array_equal(t.get_flags(), fo)
        assert (fo == 1).any() and (fo == 0).any()


@pytest.mark.parametrize("n", [16, 8])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_gradient_flags_with_non_finite_cells(amr, oracle_mod, n, dtype):
    """Infinite, NaN and huge cells (FP32 squares that overflow) next to
    ordinary ones: the lanes that hold them leave the FP32 pre-filter and
    decide exactly; flags equal the oracle's."""
    h, seed = 1, 29
    o = oracle_mod.OracleTree(2, n, h, 6, 20000)
    o.refine_all(2)
    t = amr.Tree(2, n, h, 6, capacity=20000, dtype=amr.F64 if dtype == "f64" else amr.F32)
    t.refine_uniform(2)
    o.random_state(seed)
    st = o.state()
    rng = np.random.default_rng(seed)
    P = st.shape[0]
    for p in rng.choice(P, size=P // 3, replace=False):
        y, x = rng.integers(h, n + h, size=2)
        st[p, y, x] = rng.choice([np.inf, -np.inf, np.nan, 1e30, -3e25])
    if dtype == "f32":
        st = st.astype(np.float32).astype(np.float64)
    o.set_state(st)
    o.halo_exchange()
    st = o.state()
    fo = o.flags_gradient(0.05, 0.01, 1, 4)
    t.upload_state(st)
    t.flags_gradient(0.05, 0.01, 1, 4)
    np.testing.assert_array_equal(t.get_flags(), fo)
