"""Shared helpers of the DG tests: golden fixtures (produced by running the
reference's DG patch solver, tests/golden/make_dg_golden.py) and the layout
conversion between the reference's dump ([leaf, cell, node, variable]) and
the tree's 16-field padded state."""
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ["dg_advection_l2", "dg_advection_l3", "dg_advection_l3_small_dt"]
EULER_CASES = ["dg_euler_l3"]
PATCH, FIELDS = 4, 16


def load(name):
    z = np.load(GOLDEN / f"{name}.npz")
    return {k: z[k] for k in z.files}


def leaves_to_fields(st):
    """[leaf, cell, node, var] -> [field, leaf, 6, 6] (ghosts zero)."""
    P = st.shape[0]
    out = np.zeros((FIELDS, P, PATCH + 2, PATCH + 2))
    blk = st.reshape(P, PATCH, PATCH, 4, 4)  # leaf, ly, lx, node, var
    out[:, :, 1:PATCH + 1, 1:PATCH + 1] = blk.transpose(3, 4, 0, 1, 2).reshape(FIELDS, P, PATCH, PATCH)
    return out


def fields_to_leaves(a):
    """[field, leaf, 6, 6] -> [leaf, cell, node, var] (interior cells)."""
    P = a.shape[1]
    inner = a[:, :, 1:PATCH + 1, 1:PATCH + 1].reshape(4, 4, P, PATCH, PATCH)  # node, var, leaf, ly, lx
    return inner.transpose(2, 3, 4, 0, 1).reshape(P, PATCH * PATCH, 4, 4)


def fixture_tree(name, dump):
    """(Morton ids, [leaf, cell, node, var] state) of dump `dump` of a DG
    fixture (uniform fixtures keep one id list, re-mesh fixtures one per dump)."""
    z = load(name)
    if "state" in z:
        return z["ids"], z["state"][dump]
    return z[f"ids_{dump}"], z[f"state_{dump}"]


def printer_cases():
    import json

    return json.loads((GOLDEN / "dg_vtk.json").read_text())
