"""Reader for the binary records written by oracle/ref_driver.cpp (the
reference run from its own headers).  Used by make_golden.py only."""
from __future__ import annotations

import struct

import numpy as np

TAG_TREE, TAG_FLAGS, TAG_STATE, TAG_DT = 1, 2, 3, 4

NEIGHBOR_DTYPE = np.dtype(
    [("kind", "u1"), ("quadrant", "u1", (3,)), ("pad", "<u4"), ("ids", "<u8", (4,))]
)


def read_records(path: str, rank: int):
    """Yield (tag, step, payload) tuples with payloads decoded to numpy arrays."""
    ndir = 2 * rank
    with open(path, "rb") as f:
        data = f.read()
    off = 0
    out = []
    while off < len(data):
        tag, step, nbytes = struct.unpack_from("<IIQ", data, off)
        off += 16
        body = data[off : off + nbytes]
        off += nbytes
        if tag == TAG_TREE:
            (n,) = struct.unpack_from("<Q", body, 0)
            rec = np.dtype([("id", "<u8"), ("nb", NEIGHBOR_DTYPE, (ndir,))])
            arr = np.frombuffer(body, rec, count=n, offset=8)
            out.append((tag, step, {"ids": arr["id"].copy(), "nb": arr["nb"].copy()}))
        elif tag == TAG_FLAGS:
            (n,) = struct.unpack_from("<Q", body, 0)
            out.append((tag, step, np.frombuffer(body, np.int8, count=n, offset=8).copy()))
        elif tag == TAG_STATE:
            n, flat = struct.unpack_from("<QQ", body, 0)
            out.append((tag, step, np.frombuffer(body, np.float64, count=n * flat, offset=16).reshape(n, flat).copy()))
        elif tag == TAG_DT:
            sum_dt, steps = struct.unpack_from("<dQ", body, 0)
            out.append((tag, step, (sum_dt, steps)))
        else:
            raise ValueError(f"unknown tag {tag}")
    return out
