"""Trees and states of the VTK writer fixtures (tests/golden/vtk.json): the
final tree and state of four reference fixtures, rebuilt from their flags."""
import json

import numpy as np

from conftest import GOLDEN, load_golden


def cases():
    return json.loads((GOLDEN / "vtk.json").read_text())


def rebuild(name):
    """(meta, flag sequence, padded final state, final ids, initial uniform levels)."""
    z, meta = load_golden(name)
    rank, n, h = meta["rank"], meta["n"], meta["halo"]
    P1 = n + 2 * h
    p = meta["params"]
    init = int(p["init_levels"])
    if "passes" in z.files:
        passes = int(z["passes"])
        flags = [z[f"flags_{k}"] for k in range(passes)]
        state = z[f"state_{passes - 1}"]
        ids = z[f"ids_{passes - 1}"]
    else:
        flags = []
        inner = z["state_final"]
        state = np.zeros((inner.shape[0],) + (P1,) * rank)
        state[(slice(None),) + (slice(h, n + h),) * rank] = inner
        ids = z["final_ids"]
    return meta, flags, state, ids, init
