"""Data-parallel training of the warm-start network: one gradient all-reduce per step.

Every rank holds the whole network and trains on its own share of the
simulated scans (``shard``).  After each rank's backward pass has filled the
parameter gradients, ``GradientAllReduce`` sums them over the ranks in one
collective on one flat buffer (coalesced, so a step costs one all-reduce
rather than one per tensor) and divides by the number of ranks.  Each rank's
loss is a mean over an equal share of the global batch, so the result is the
gradient of the global batch's mean loss and every rank's Adam step is the
same.  The collective is whatever ``torch.distributed`` was initialised with:
NCCL for CUDA gradients, gloo for CPU tensors.

Nothing in the plain reconstruction needs this: a scan is a sequential chain
(each position reads the previous position's probe and object), so scans run
as independent replicas; only the network's training has an exchange step.
"""

from __future__ import annotations


def _dist():
    import torch.distributed as dist

    return dist


def world():
    """(rank, world size) of the initialised process group, or (0, 1)."""
    dist = _dist()
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(), dist.get_world_size()
    return 0, 1


def shard(items, rank=None, world_size=None):
    """This rank's share of a list of training scans (round robin)."""
    if rank is None or world_size is None:
        rank, world_size = world()
    return list(items)[rank::world_size]


class GradientAllReduce:
    """Average a fixed list of gradient tensors over the ranks, in place.

    ``tensors`` must keep their storage across steps (the network's ``.g``
    buffers do); they are copied into one flat buffer of their common dtype
    and device, reduced with one ``all_reduce`` and copied back."""

    def __init__(self, tensors, group=None, average=True):
        import torch

        self.tensors = list(tensors)
        if not self.tensors:
            raise ValueError("GradientAllReduce needs at least one tensor")
        dt, dev = self.tensors[0].dtype, self.tensors[0].device
        if any(t.dtype != dt or t.device != dev for t in self.tensors):
            raise ValueError("GradientAllReduce: all tensors must share dtype and device")
        self.group = group
        self.average = average
        self.sizes = [t.numel() for t in self.tensors]
        self.flat = torch.empty(sum(self.sizes), dtype=dt, device=dev)

    def __call__(self):
        dist = _dist()
        if not (dist.is_available() and dist.is_initialized()):
            return
        n = dist.get_world_size(self.group)
        if n == 1:
            return
        off = 0
        for t, k in zip(self.tensors, self.sizes):
            self.flat[off : off + k].copy_(t.reshape(-1))
            off += k
        dist.all_reduce(self.flat, op=dist.ReduceOp.SUM, group=self.group)
        if self.average:
            self.flat.div_(n)
        off = 0
        for t, k in zip(self.tensors, self.sizes):
            t.copy_(self.flat[off : off + k].view(t.shape))
            off += k


def network_reducer(net, group=None):
    """GradientAllReduce over every parameter gradient of a WarmStartNet."""
    return GradientAllReduce([p.g for p in net.parameters()], group=group)
