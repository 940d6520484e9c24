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


def _grad_worker(rank, world, port, q):
    """Each rank: the oracle network's parameter gradients on its half of a
    batch, averaged over the ranks by the package's all-reduce."""
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import torch
    import torch.distributed as dist

    from oracle import nn_oracle as N
    from ptylab_gb300.warmstart.dataparallel import GradientAllReduce, shard

    dist.init_process_group("gloo", rank=rank, world_size=world)
    params = N.init_params(seed=3, levels=(8, 16, 16, 16))
    rng = np.random.default_rng(7)
    batch = rng.standard_normal((4, 16, 16, 1))
    target = rng.standard_normal((4, 16, 16, 2))
    mine = np.stack(shard(list(batch), rank, world))
    tmine = np.stack(shard(list(target), rank, world))
    net = N.Net(params)
    out = net.forward(mine)
    g = net.backward((out - tmine) / out.size)  # gradient of this rank's mean squared loss / 2
    names = sorted(g)
    grads = [torch.from_numpy(np.ascontiguousarray(a)) for n in names for a in g[n]]
    GradientAllReduce(grads)()
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, [t.numpy() for t in grads]))


def test_two_gloo_ranks_average_network_gradients():
    """Data-parallel training's one exchange step: the averaged per-rank
    gradients equal the gradient of the whole batch's mean loss."""
    import numpy as np

    sys.path.insert(0, str(ROOT))
    from oracle import nn_oracle as N

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29600 + os.getpid() % 1000
    procs = [ctx.Process(target=_grad_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    params = N.init_params(seed=3, levels=(8, 16, 16, 16))
    rng = np.random.default_rng(7)
    batch = rng.standard_normal((4, 16, 16, 1))
    target = rng.standard_normal((4, 16, 16, 2))
    net = N.Net(params)
    o = net.forward(batch)
    g = net.backward((o - target) / o.size)  # whole-batch mean loss = the average of the halves' means
    want = [a for n in sorted(g) for a in g[n]]
    for r in (0, 1):
        assert len(out[r]) == len(want)
        for a, b in zip(out[r], want):
            np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-12)
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)
