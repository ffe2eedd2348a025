"""The device-resident VTK writer (amr_tree_write_vtk) against the reference
writer's files (SHA-256 and length from the reference build,
tests/golden/vtk.json) on the final tree and state of six fixtures (2D,
3D, halo 2, the Euler fields on a 1000-long domain): byte-identical."""
import hashlib

import numpy as np
import pytest

from vtk_cases import cases, fields, lengths, rebuild

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(cases()))
def test_gpu_vtk_matches_reference(tmp_path, name):
    import amr_gb300 as A

    want = cases()[name]
    meta, flags, state, ids, init = rebuild(name)
    nvar = fields(meta)
    t = A.Tree(meta["rank"], meta["n"], meta["halo"], meta["depth"], capacity=20000, fields=nvar,
               lengths=lengths(meta, meta["rank"]))
    t.refine_uniform(init)
    for f in flags:
        t.set_flags(f)
        t.remesh()
    np.testing.assert_array_equal(t.ids(), ids)
    t.upload_state(np.moveaxis(state, 1, 0) if nvar > 1 else state)
    path = tmp_path / f"{name}.vtk"
    t.write_vtk(path, want["field"])
    data = path.read_bytes()
    assert len(data) == want["bytes"]
    assert hashlib.sha256(data).hexdigest() == want["sha256"]


def test_gpu_vtk_fp32_tree_writes_float_values(tmp_path):
    """An FP32 tree writes its values as "float" (4 bytes, big-endian); the
    geometry sections are those of the FP64 file."""
    import amr_gb300 as A

    name = "tree_random_2d_n8"
    meta, flags, state, ids, init = rebuild(name)
    files = {}
    for dt in (A.F64, A.F32):
        t = A.Tree(meta["rank"], meta["n"], meta["halo"], meta["depth"], capacity=20000, dtype=dt)
        t.refine_uniform(init)
        for f in flags:
            t.set_flags(f)
            t.remesh()
        t.upload_state(state)
        p = tmp_path / f"{dt}.vtk"
        t.write_vtk(p)
        files[dt] = p.read_bytes()
    a, b = files[A.F64], files[A.F32]
    cut = a.index(b"SCALARS Scalar double 1\n")
    assert b[:cut] == a[:cut]
    tail = b[cut:].split(b"LOOKUP_TABLE default\n", 1)[1]
    n_cells = len(ids) * meta["n"] ** meta["rank"]
    assert len(tail) == 4 * n_cells
    vals = np.frombuffer(tail, ">f4")
    ref = np.frombuffer(a[cut:].split(b"LOOKUP_TABLE default\n", 1)[1], ">f8")
    np.testing.assert_array_equal(vals, ref.astype(np.float32))
