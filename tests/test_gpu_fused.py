"""The fused interval kernel (k_run_interval2d: ten update steps and the
gradient flags of a re-mesh interval in one pass over 4x4-patch blocks)
through amr_tree_run, against the per-leaf kernels of the same interval
(multi-step passes and the uniform flag kernel, AMR_RUN_NO_FUSED).

The fused kernel applies the same update operation to the same inputs as
one-step launches (packed FP32 operations round per component like the
scalar ones) and evaluates the same gradient rule on the same ghost values,
so the bar is bit-identity: interior state, leaves, levels, flags and the
per-instance time, on static forests and on forests whose flags re-mesh
them after the first interval.  The FP32 result is also held to the FP64
oracle (relative L2 <= 1e-5 per instance).
"""
import numpy as np
import pytest

from conftest import interior, rel_l2

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5
N, DEPTH, CFL = 16, 7, 0.4


@pytest.fixture(scope="module")
def amr():
    import amr_gb300 as A

    A.lib()
    return A


def _forest(A, caps, vels, bounds, seed):
    K = len(caps)
    cap = int(sum(4 ** int(c) for c in caps)) * 4 + 64
    f = A.Tree(2, N, 1, DEPTH, capacity=cap, dtype=A.F32, instances=K)
    f.refine_to_levels(caps)
    off = f.instance_offsets()
    rng = np.random.default_rng(seed)
    y, x = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    st = []
    for i in range(K):
        P = off[i + 1] - off[i]
        u = np.zeros((P, N + 2, N + 2))
        # smooth waves plus small noise: gradients above and below both thresholds
        for p in range(P):
            u[p, 1:N + 1, 1:N + 1] = np.sin(0.3 * (x + p)) * np.cos(0.2 * (y - p)) + 1e-3 * rng.standard_normal((N, N))
        st.append(u)
    f.upload_state(np.concatenate(st).astype(np.float32))
    f.set_instance_params(velocity=vels, level_bounds=bounds)
    return f


def _run(f, steps, fused):
    return f.run(steps, 10, None, CFL, "grad", 0.05, 0.01, fused=fused)


def _same(a, b, nflags):
    """Bit-identity of two runs; the flags of the last interval are compared
    on the nflags leaves it flagged (entries past them were not written)."""
    np.testing.assert_array_equal(a.ids(), b.ids())
    np.testing.assert_array_equal(a.levels(), b.levels())
    np.testing.assert_array_equal(interior(a.download_state(), 2, N, 1), interior(b.download_state(), 2, N, 1))
    if nflags:
        np.testing.assert_array_equal(a.get_flags()[:nflags], b.get_flags()[:nflags])
    ta, ca = a.instance_time()
    tb, cb = b.instance_time()
    np.testing.assert_array_equal(ta, tb)
    np.testing.assert_array_equal(ca, cb)


# every sign combination of the velocity, zero components included, and
# instances of one block (level 2, the halo wraps onto the block itself) up
# to 8 x 8 blocks
CAPS = [2, 3, 2, 4, 2, 3, 5, 2, 3]
VELS = [(1.0, 0.5), (-0.7, 0.3), (0.2, -1.0), (-0.5, -0.5), (0.0, 0.8), (0.9, 0.0), (-0.3, 0.6), (0.0, -0.4),
        (-1.0, 0.0)]


def test_fused_static_forest_equals_per_leaf_kernels(amr):
    """Static caps (min = max level): three fused intervals equal three
    intervals of multi-step passes and the flag kernel bit for bit."""
    bounds = [(c, c) for c in CAPS]
    a = _forest(amr, CAPS, VELS, bounds, 1)
    b = _forest(amr, CAPS, VELS, bounds, 1)
    sa = _run(a, 30, True)
    sb = _run(b, 30, False)
    assert sa["graph_intervals"] == sb["graph_intervals"] == 3
    assert sa["cell_updates"] == sb["cell_updates"]
    _same(a, b, len(a.ids()))


def test_fused_flags_drive_the_same_remesh(amr):
    """Bounds that let every instance refine and coarsen: the fused
    interval's flags re-mesh the forest exactly as the flag kernel's do (the
    later intervals, on the adapted forest, run the per-leaf kernels)."""
    bounds = [(max(0, c - 1), c + 1) for c in CAPS]
    for steps in (10, 40):
        a = _forest(amr, CAPS, VELS, bounds, 2)
        b = _forest(amr, CAPS, VELS, bounds, 2)
        ids0 = a.ids()
        sa = _run(a, steps, True)
        sb = _run(b, steps, False)
        assert len(a.ids()) != len(ids0) or not np.array_equal(a.ids(), ids0)  # the flags changed the forest
        assert sa["leaves_max"] == sb["leaves_max"] and sa["cell_updates"] == sb["cell_updates"]
        # one interval: its flags are the fused kernel's (on the initial leaves)
        _same(a, b, len(ids0) if steps == 10 else 0)


def test_fused_timed_launches_equal_graph_replay(amr):
    """With per-launch timing the interval's kernels are issued directly
    (CUDA events around the fused kernel): same result as the graph."""
    bounds = [(c, c) for c in CAPS]
    a = _forest(amr, CAPS, VELS, bounds, 3)
    b = _forest(amr, CAPS, VELS, bounds, 3)
    a.set_timing(True)
    _run(a, 20, True)
    ms, launches, cells = a.get_timing()
    a.set_timing(False)
    _run(b, 20, True)
    assert launches == 2 and ms > 0.0
    assert cells == 2 * 10 * len(a.ids()) * N * N
    _same(a, b, len(a.ids()))


def test_fused_guard_falls_back_on_small_instances(amr):
    """An instance below level 2 (fewer than 16 leaves) is not made of 4x4
    blocks: the guard stops the fused interval before any work and the run
    continues with the per-leaf kernels, with the same result."""
    caps = [2, 1, 3]
    vels = VELS[:3]
    bounds = [(c, c) for c in caps]
    a = _forest(amr, caps, vels, bounds, 4)
    b = _forest(amr, caps, vels, bounds, 4)
    _run(a, 20, True)
    _run(b, 20, False)
    _same(a, b, len(a.ids()))


def test_fused_forest_against_fp64_oracle(amr, oracle_mod):
    """Fused FP32 intervals against the FP64 oracle run of each instance:
    the trees equal, the state within 1e-5 relative L2, the time exact."""
    O = oracle_mod
    caps = [2, 3, 2, 4]
    vels = VELS[:4]
    bounds = [(c, c) for c in caps]
    f = _forest(amr, caps, vels, bounds, 5)
    s0 = f.download_state().astype(np.float64)
    off = f.instance_offsets()
    st = _run(f, 30, True)
    assert st["graph_intervals"] == 3
    s = interior(f.download_state(), 2, N, 1)
    acc, _ = f.instance_time()
    for i, cap in enumerate(caps):
        o = O.OracleTree(2, N, 1, DEPTH, 20000)
        o.refine_all(cap)
        o.set_state(s0[off[i]:off[i + 1]])
        o.halo_exchange()
        sum_dt = 0.0
        for _ in range(3):
            a, _ = o.advance(10, vels[i], CFL)
            sum_dt += a
            fl = o.flags_gradient(0.05, 0.01, cap, cap)
            assert o.reconstruct(fl) == 0
            o.halo_exchange()
        ids = f.ids()[off[i]:off[i + 1]] & np.uint64((1 << (6 + 2 * DEPTH)) - 1)
        np.testing.assert_array_equal(ids, o.ids())
        assert rel_l2(s[off[i]:off[i + 1]], interior(o.state(), 2, N, 1)) <= FP32_TOL, i
        assert acc[i] == sum_dt
