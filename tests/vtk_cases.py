"""Trees and states of the VTK writer fixtures (tests/golden/vtk.json): the
final tree and state of six reference fixtures (four scalar, two Euler),
rebuilt from their flags."""
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
    if "remeshes" in z.files:  # Euler fixtures: (size, nvar, ...) states
        k = int(z["remeshes"])
        flags = [z[f"flags_{i}"] for i in range(k)]
        state = z["state_final"]
        ids = z[f"ids_{k - 1}"]
    elif "passes" in z.files:
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


def fields(meta):
    return int(meta.get("nvar", 1))


def lengths(meta, rank):
    return tuple(meta.get("lengths", [1.0] * rank))
