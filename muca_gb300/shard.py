"""Host-side sharding of chains over processes.

The reference runs one chain set per GPU of starting_gpu..last_gpu, each with
its own seeds, and sums the per-GPU histograms on the host after every
iteration (muca_delta_multigpu.cu:404-429).  Here a process (rank) owns a
contiguous range of those reference devices; `reduce_histogram` is the
per-iteration sum across ranks (torch.distributed, any backend), and
`max_over_ranks` gives the job time of a timed region.
"""
from __future__ import annotations

import numpy as np


def shard_devices(world_size: int, rank: int, ndev_total: int):
    """(dev_offset, ndev) of `rank`: reference devices split as evenly as
    possible, lower ranks taking the remainder."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("bad rank %d of %d" % (rank, world_size))
    if ndev_total < world_size:
        raise ValueError("%d devices cannot be shared by %d ranks" % (ndev_total, world_size))
    base, extra = divmod(ndev_total, world_size)
    off = rank * base + min(rank, extra)
    return off, base + (1 if rank < extra else 0)


def reduce_histogram(h: np.ndarray, group=None) -> np.ndarray:
    """Sum of the ranks' u64 histograms (returned on every rank)."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(h).view(np.int64).copy())
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.numpy().view(np.uint64)


def max_over_ranks(x: float, group=None) -> float:
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
