"""The oracle's VTK writer against the reference's (include/ndtree/
vtk_print.hpp) on six fixtures (scalar and Euler): the files must be byte-identical (SHA-256
and length recorded from the reference build)."""
import hashlib

import numpy as np
import pytest

from vtk_cases import cases, fields, lengths, rebuild


@pytest.mark.parametrize("name", sorted(cases()))
def test_oracle_vtk_matches_reference(oracle_mod, tmp_path, name):
    want = cases()[name]
    meta, flags, state, ids, init = rebuild(name)
    t = oracle_mod.OracleTree(meta["rank"], meta["n"], meta["halo"], meta["depth"], 20000, nvar=fields(meta),
                              lengths=lengths(meta, meta["rank"]))
    t.refine_all(init)
    for f in flags:
        assert t.reconstruct(f) == 0
    np.testing.assert_array_equal(t.ids(), ids)
    t.set_state(state)
    path = tmp_path / f"{name}.vtk"
    t.write_vtk(path, want["field"])
    data = path.read_bytes()
    assert len(data) == want["bytes"]
    assert hashlib.sha256(data).hexdigest() == want["sha256"]
