"""The bench's multi-rank path (replicas only: no data-path collective) on
CPU: two gloo ranks run the aggregation that `bench.py --gpus 2` runs over
NCCL — max of the times, sum of the cell updates."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: (r+1) * 10 ms, (r+1) * 1000 cell updates
        res = bench.aggregate_replicas(torch, "cpu", 10.0 * (rank + 1), 20.0 * (rank + 1), 1000 * (rank + 1),
                                       500 * (rank + 1))
        out[rank] = res
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    port = _free_port()
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        ms, e2e_ms, cells, e2e_cells = res[r]
        assert (ms, e2e_ms) == (20.0, 40.0)
        assert (cells, e2e_cells) == (3000.0, 1500.0)
