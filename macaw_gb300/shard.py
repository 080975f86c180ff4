"""History sharding across ranks, one process per GPU.

Histories are independent and each one's random numbers are keyed by its
global particle id, so a fixed-source run shards by contiguous ranges of
history indices with no exchange while tracking; the one exchange step is
an FP64 sum of the element tallies at the end.  The reference keeps its
tallies per MPI rank and lets OpenMC reduce them
(src/userobjects/OpenMCStudy.C:391-396); here the sum goes through
torch.distributed (NCCL between GPUs, gloo on the host).
"""
from __future__ import annotations

import numpy as np


def history_range(n_total: int, rank: int, world: int) -> tuple[int, int]:
    """(first, count) of rank's share of histories 0..n_total-1: contiguous,
    the remainder spread one each over the lowest ranks."""
    if world < 1 or not 0 <= rank < world or n_total < 0:
        raise ValueError("bad rank/world/history count")
    base, extra = divmod(n_total, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def reduce_tally(tally, group=None):
    """Sums an FP64 tally over every rank of the default (or given) process
    group and returns the sum (a numpy array for a numpy input, else the
    tensor, reduced in place).  With one rank, or without an initialised
    group, the tally is returned as it is."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return tally
    as_numpy = isinstance(tally, np.ndarray)
    t = torch.from_numpy(np.ascontiguousarray(tally, np.float64)) if as_numpy else tally
    if t.dtype != torch.float64:
        raise TypeError("tallies are summed in float64")
    dev = t
    if dist.get_backend(group) == "nccl" and not t.is_cuda:
        dev = t.cuda()
    dist.all_reduce(dev, op=dist.ReduceOp.SUM, group=group)
    if dev is not t:
        t.copy_(dev.cpu())
    return t.numpy() if as_numpy else t
