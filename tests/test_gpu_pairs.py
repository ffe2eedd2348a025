"""Two update steps per pass over memory (trees whose every neighbour relation
is same-level): bit-identical to the same steps taken one launch at a time.

* host-driven advance: advance(k) (passes of two steps, an odd last step
  alone) against k calls of advance(1), FP32 and FP64, 16x16 and 8x8
  patches, every combination of upwind sides including zero velocity
  components;
* graph path of amr_tree_run on a forest with per-instance velocities held
  at its caps: re-mesh interval 10 (passes) against interval 1 (one step per
  interval): states bit-identical;
* a forest that becomes non-uniform at its first re-mesh: the guarded graph
  interval stops before it runs and the run continues one step at a time;
  graph and host-driven runs agree bit for bit and match the oracle
  (tests/test_gpu_forest.py holds the oracle comparison).
"""
import numpy as np
import pytest

from conftest import interior

pytestmark = pytest.mark.gpu

VELS = [(1.0, 0.5), (-0.7, 0.3), (0.2, -1.0), (-0.5, -0.5), (0.0, 0.8), (0.9, 0.0), (0.0, -1.0), (-1.0, 0.0)]


@pytest.fixture(scope="module")
def amr():
    import amr_gb300 as A

    A.lib()
    return A


def _tree(amr, n, dtype, state):
    t = amr.Tree(2, n, 1, 6, capacity=4096, dtype=dtype)
    t.refine_uniform(3)
    t.upload_state(state)
    return t


@pytest.mark.parametrize("n", [16, 8])
@pytest.mark.parametrize("dtype", ["F32", "F64"])
@pytest.mark.parametrize("vel", VELS)
def test_pair_passes_equal_single_steps(amr, n, dtype, vel):
    dt = getattr(amr, dtype)
    rng = np.random.default_rng(1000 * n + 10 * VELS.index(vel) + (dtype == "F64"))
    state = rng.standard_normal((64, n + 2, n + 2))
    a = _tree(amr, n, dt, state)
    a.advance(7, vel, 0.4)
    acc_a, ex_a = a.finish_advance()
    b = _tree(amr, n, dt, state)
    acc_b = 0.0
    for _ in range(7):
        b.advance(1, vel, 0.4)
        acc, ex = b.finish_advance()
        acc_b += acc
    assert ex_a == 7
    assert abs(acc_a - acc_b) <= 1e-15 * acc_a
    np.testing.assert_array_equal(interior(a.download_state(), 2, n, 1), interior(b.download_state(), 2, n, 1))


def test_forest_graph_passes_equal_one_step_intervals(amr):
    import amr_gb300 as A

    caps = [1, 2, 3, 2, 1, 2, 3, 1]
    K = len(caps)
    vel = [VELS[i % len(VELS)] for i in range(K)]
    res = []
    for interval in (10, 1):
        f = amr.Tree(2, 16, 1, 5, capacity=8192, dtype=amr.F32, instances=K)
        f.refine_to_levels(caps)
        f.set_instance_params(velocity=vel, level_bounds=[(c, c) for c in caps])
        rng = np.random.default_rng(5)
        f.upload_state(rng.standard_normal((f.size, 18, 18)).astype(np.float32))
        st = f.run(40, interval, None, 0.4, "grad", 0.05, 0.01)
        assert st["executed_steps"] == 40 and st["graph_intervals"] == st["intervals"]
        res.append(interior(f.download_state(), 2, 16, 1))
    np.testing.assert_array_equal(res[0], res[1])


@pytest.mark.parametrize("n", [16, 8])
@pytest.mark.parametrize("dtype", ["F64", "F32"])
def test_forest_turning_non_uniform_graph_equals_host(amr, n, dtype):
    """Uniform at the start (each instance at its cap), refinement allowed:
    the first interval's flags come from the same-level flag kernel (face
    records), the host-driven run's from the general one; after the first
    re-mesh the tree has coarse-fine faces, the next guarded interval stops
    and the run goes on with one-step intervals.  Meshes and states agree
    bit for bit."""
    import amr_gb300 as A

    caps = [1, 2, 2, 1]
    K = len(caps)
    out = []
    for graph in (True, False):
        f = amr.Tree(2, n, 1, 5, capacity=20000, dtype=getattr(amr, dtype), instances=K)
        f.refine_to_levels(caps)
        f.set_instance_params(velocity=VELS[:K], level_bounds=[(0, 4)] * K)
        b = [A.seeded_bumps(2, 2, 40 + i, sigma=(0.04, 0.08), amp=(0.5, 2.0)) for i in range(K)]
        off = f.instance_offsets()
        ids = f.ids()
        st0 = np.concatenate([A.gaussian_state(ids[off[i]:off[i + 1]], 2, n, 1, 5, b[i]) for i in range(K)])
        if dtype == "F32":
            st0 = st0.astype(np.float32)
        f.upload_state(st0)
        st = f.run(30, 10, None, 0.4, "grad", 0.05, 0.01, graph=graph)
        assert st["executed_steps"] == 30
        out.append((f.ids(), interior(f.download_state(), 2, n, 1), st["remeshes"], st["graph_intervals"]))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2] == 3
    assert out[0][3] >= 1 and out[1][3] == 0


@pytest.mark.parametrize("dtype", ["F32", "F64"])
def test_uniform_flags_equal_general_flags(amr, dtype):
    """A forest held uniform (each instance refined to its cap, bounds one
    level either side so refine and coarsen decisions both occur): one graph
    interval (pass records, same-level flag kernel) against the host-driven
    interval (general flag kernel) gives the same re-mesh."""
    import amr_gb300 as A

    caps = [2, 3, 3, 2, 3, 2]
    K = len(caps)
    out = []
    for graph in (True, False):
        f = amr.Tree(2, 16, 1, 5, capacity=40000, dtype=getattr(amr, dtype), instances=K)
        f.refine_to_levels(caps)
        f.set_instance_params(velocity=[VELS[(3 * i) % len(VELS)] for i in range(K)],
                              level_bounds=[(c - 1, c + 1) for c in caps])
        b = [A.seeded_bumps(2, 3, 70 + i, sigma=(0.03, 0.09), amp=(0.2, 2.0)) for i in range(K)]
        off = f.instance_offsets()
        ids = f.ids()
        st0 = np.concatenate([A.gaussian_state(ids[off[i]:off[i + 1]], 2, 16, 1, 5, b[i]) for i in range(K)])
        if dtype == "F32":
            st0 = st0.astype(np.float32)
        f.upload_state(st0)
        st = f.run(10, 10, None, 0.4, "grad", 0.05, 0.01, graph=graph)
        assert st["executed_steps"] == 10 and st["remeshes"] == 1
        out.append((f.ids(), interior(f.download_state(), 2, 16, 1)))
    assert len(out[0][0]) != sum(4 ** c for c in caps)  # the re-mesh changed the tree
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
