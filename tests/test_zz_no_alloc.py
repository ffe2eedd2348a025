"""amr_remesh_noalloc: the allocation-free re-mesh for callers that cannot call
cudaMalloc (code that runs inside a memory pool or arena it does not own, or
a process whose device allocator is locked).  It must give the same tree,
neighbour tables and state as the tree's own re-mesh (amr_tree_remesh), on two
calls in a row, with the second call fed the first call's output.

This file runs last (conftest.py orders it after the end-to-end tests), so
that a run stopping at its first failure has run every other test before
it."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-12  # the same bar as the other FP64 state tests


def _noalloc(A, geom, ids, meta, flags, state, out_cap):
    import torch

    dev = torch.device("cuda:0")
    n = ids.size
    t_ids = torch.from_numpy(ids.view(np.int64)).to(dev)
    t_meta = torch.from_numpy(meta.view(np.uint8).reshape(-1)).to(dev)
    t_flags = torch.from_numpy(flags.astype(np.int8)).to(dev)
    t_state = torch.from_numpy(np.ascontiguousarray(state, np.float64)).to(dev)
    o_ids = torch.zeros(out_cap, dtype=torch.int64, device=dev)
    o_lev = torch.zeros(out_cap, dtype=torch.int32, device=dev)
    o_meta = torch.zeros(out_cap * meta.shape[1] * A.HALO_META.itemsize, dtype=torch.uint8, device=dev)
    o_state = torch.zeros((out_cap,) + state.shape[1:], dtype=torch.float64, device=dev)
    o_count = torch.zeros(1, dtype=torch.int32, device=dev)
    host_count = C.c_size_t(0)
    L = A.lib()
    L.amr_remesh_noalloc.argtypes = [C.POINTER(A.PatchGeometry), C.c_size_t] + [C.c_void_p] * 4 + [C.c_size_t] + \
        [C.c_void_p] * 5 + [C.POINTER(C.c_size_t), C.c_void_p]
    A.check(L.amr_remesh_noalloc(C.byref(geom), n, t_ids.data_ptr(), t_meta.data_ptr(), t_flags.data_ptr(),
                                 t_state.data_ptr(), out_cap, o_ids.data_ptr(), o_lev.data_ptr(), o_meta.data_ptr(),
                                 o_state.data_ptr(), o_count.data_ptr(), C.byref(host_count),
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    m = host_count.value
    assert int(o_count.item()) == m
    ids_o = o_ids[:m].cpu().numpy().view(np.uint64)
    lev_o = o_lev[:m].cpu().numpy()
    meta_o = o_meta.cpu().numpy()[: m * meta.shape[1] * A.HALO_META.itemsize].view(A.HALO_META).reshape(m, -1)
    state_o = o_state[:m].cpu().numpy()
    return ids_o, lev_o, meta_o, state_o


@pytest.mark.parametrize("rank,n,levels", [(2, 8, 2), (3, 4, 1)])
def test_noalloc_remesh_matches_tree_remesh(rank, n, levels):
    pytest.importorskip("torch")
    import amr_gb300 as A

    rng = np.random.default_rng(7)
    h = 1
    tree = A.Tree(rank, n, h, 7, capacity=20000)
    tree.refine_uniform(levels)
    tree.upload_state(rng.standard_normal((tree.size,) + (n + 2 * h,) * rank))
    geom = A.geometry(rank, n, h, 7)
    sl = (slice(None),) + (slice(h, n + h),) * rank

    ids, meta, state = tree.ids(), tree.neighbors(), tree.download_state()
    for call in range(2):  # two calls in a row, the second on the first's output
        flags = rng.choice(np.array([0, 1, 2], np.int8), size=ids.size, p=[0.5, 0.25, 0.25])
        if call == 1:
            flags[:] = np.where(rng.random(ids.size) < 0.7, 2, flags)  # let whole sibling groups coarsen
        got_ids, got_lev, got_meta, got_state = _noalloc(A, geom, ids, meta, flags, state, out_cap=20000)
        tree.set_flags(flags)
        tree.remesh()
        np.testing.assert_array_equal(got_ids, tree.ids())
        np.testing.assert_array_equal(got_lev, tree.levels())
        want_meta = tree.neighbors()
        for field in ("relation", "neighbor", "finer_ids", "quadrant"):
            np.testing.assert_array_equal(got_meta[field], want_meta[field])
        want_state = tree.download_state()
        den = np.linalg.norm(want_state[sl])
        assert np.linalg.norm(got_state[sl] - want_state[sl]) / den <= STATE_TOL
        ids, meta, state = got_ids, got_meta, got_state


def test_noalloc_rejects_oversized_input():
    import amr_gb300 as A

    L = A.lib()
    L.amr_remesh_noalloc.argtypes = [C.POINTER(A.PatchGeometry), C.c_size_t] + [C.c_void_p] * 4 + [C.c_size_t] + \
        [C.c_void_p] * 5 + [C.POINTER(C.c_size_t), C.c_void_p]
    geom = A.geometry(2, 8, 1, 7)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    code = L.amr_remesh_noalloc(C.byref(geom), 65537, dummy, dummy, dummy, dummy, 100, dummy, dummy, dummy, dummy,
                                dummy, None, None)
    assert code == A.AMR_ERR_INVALID
    assert b"AMR_NOALLOC_MAX_LEAVES" in L.amr_last_error()
