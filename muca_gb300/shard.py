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


def next_nupdates(nup: int, full: bool, covered: bool, sched: int, cap: int) -> int:
    """The NUPDATES schedule of the device-side run (k_weights.cu
    next_nupdates): 0 the reference's (NUP+1)*1.01 once the width is full
    (muca_delta_multigpu.cu:379-382), 1 doubling once full, 2 doubling every
    iteration, 3 as 0 and doubling once every bin holds >= 5 % of the mean,
    4 NUP*1.05 every iteration (muca_mag.cpp:131); `cap` 0 = none (2^30 for
    the doubling schedules and 4), never below the current value."""
    nx = nup
    if sched == 2 or (sched == 1 and full) or (sched == 3 and full and covered):
        nx = 2 * nup
        cap = cap or (1 << 30)
    elif sched in (0, 3) and full:
        nx = int((nup + 1) * 1.01)
    elif sched == 4:
        nx = int(nup * 1.05)
        cap = cap or (1 << 30)
    if cap and nx > cap:
        nx = cap if cap > nup else nup
    return nx & 0xFFFFFFFF


def weight_run_sharded(eng, nchains_total: int, starting_M=1, rule=0, flat_minmean=0, max_iter=1000000,
                       nup_schedule=0, nup_max=0, min_over_mean=0.5, d_kl_max=1e-4, therm=None, width_start=0,
                       hold_until_full=0, group=None):
    """The reference's multi-GPU weight loop (muca_delta_multigpu.cu:374-477)
    over processes: every rank sweeps the chains of its own reference devices
    (`eng`, a context with that rank's dev_offset and ndev, chains already
    initialised), the ranks sum their histograms (`reduce_histogram`, the
    host sum of :404-429), and every rank takes the statistics and the FP64
    update of the same summed histogram, so the weights stay identical on all
    ranks without a broadcast.  The bookkeeping (running width, convergence,
    NUPDATES) is the device-side run's (k_weights.cu), step for step, so one
    rank with all devices reproduces muca_weight_run.  `nchains_total`: the
    chains of all ranks (acc_NUP counts them).  Without an initialised
    process group the sum is the rank's own histogram.

    `eng` needs N and sweep / histogram / set_histogram / hist_stats /
    update_weights as muca_gb300.Engine has them.  Returns a dict with
    iterations, converged, total_run and width_reached_iter."""
    import torch.distributed as dist
    N = eng.N
    multi = dist.is_available() and dist.is_initialized()
    width = width_start or 10
    nup = int(starting_M)
    if nup_schedule == 4:
        nup = next_nupdates(nup, False, False, 4, nup_max)
    elif width == N and nup_schedule != 2:
        nup = next_nupdates(nup, True, False, 1 if nup_schedule == 1 else 0, nup_max)
    total_run = nup * nchains_total
    therm = N if therm is None else therm
    k, reach_k, converged = 0, None, False
    while True:
        eng.sweep(k, 100, 1000, therm, nup)  # seed SEED + 1000 * device (:393)
        if multi:
            eng.set_histogram(reduce_histogram(eng.histogram(), group))
        s = eng.hist_stats()
        width = max(width, s.end - s.start)
        if width == N and reach_k is None:
            reach_k = k
        conv = (s.min_over_mean >= min_over_mean) if flat_minmean else (width == N and s.d_kl < d_kl_max)
        if conv:
            converged = True
            break
        if not hold_until_full or width == N:
            eng.update_weights(rule)
        k += 1
        if k >= max_iter:
            break
        nup = next_nupdates(nup, width == N, s.min_over_mean >= 0.05, nup_schedule, nup_max)
        total_run += nup * nchains_total
    return {"iterations": k + 1 if converged else k, "converged": converged, "total_run": total_run,
            "width_reached_iter": reach_k}
