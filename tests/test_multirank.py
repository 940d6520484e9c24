"""bench.py's multi-rank path on CPU: two gloo ranks (127.0.0.1) reduce the
timed region to the slowest rank and the units to the whole job."""

import os
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    t, u = bench.reduce_over_ranks(1.0 + rank, 100 * (rank + 1))
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, u))


def test_two_gloo_ranks_reduce_time_and_units():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2.0, 300.0), (1, 2.0, 300.0)]


def test_single_process_reduction_is_identity():
    import bench

    assert bench.reduce_over_ranks(3.5, 42) == (3.5, 42.0)
