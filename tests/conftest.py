import json
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
GOLDEN = REPO / "tests" / "golden"
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "gpu-amr_gb300"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "endtoend: a whole solver loop or output file; runs after every other test")


def pytest_collection_modifyitems(config, items):
    """End-to-end tests (whole solver loops, output files) run after the unit
    and parity tests, and the allocation-free re-mesh test (its own file)
    after everything, so that a run stopping at its first failure has run
    every other test before it."""
    items.sort(key=lambda item: (item.path.name == "test_zz_no_alloc.py",
                                 item.get_closest_marker("endtoend") is not None))


def load_golden(name):
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(z["meta"]))
    return z, meta


def bumps_of(meta):
    s = str(meta["params"].get("bumps", ""))
    return [float(x) for x in s.replace(";", ",").split(",") if x]


def vel_of(meta):
    return [float(x) for x in str(meta["params"]["vel"]).split(",")]


def interior(state, rank, n, h):
    sl = (slice(None),) + (slice(h, n + h),) * rank
    return state[sl]


def face_mask(rank, n, h):
    """Interior plus face-ghost cells (corners/edges of the ghost layer are
    never written by the reference's face-only halo exchange)."""
    P1 = n + 2 * h
    g = np.indices((P1,) * rank)
    inside = (g >= h) & (g < n + h)
    return (~inside).sum(0) <= 1


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def neighbors_linear(ids, nb, rank):
    """Oracle neighbour records (Morton ids) -> (kind, linear ids, quadrant)
    in the golden layout."""
    pos = {int(k): i for i, k in enumerate(ids)}
    kind = nb["kind"].astype(np.int8)
    nbid = np.full(nb["ids"].shape, -1, np.int32)
    nf = 2 ** (rank - 1)
    P, D, _ = nbid.shape
    for p in range(P):
        for d in range(D):
            k = kind[p, d]
            if k in (1, 3):
                nbid[p, d, 0] = pos[int(nb["ids"][p, d, 0])]
            elif k == 2:
                for f in range(nf):
                    nbid[p, d, f] = pos[int(nb["ids"][p, d, f])]
    quad = nb["quadrant"].astype(np.int8)
    quad[kind != 3] = 0
    return kind, nbid, quad


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O

    O.build()
    return O
