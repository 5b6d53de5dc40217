"""Sharding of reference devices over processes, on CPU with gloo (2 ranks):
each rank runs its devices' chains (the oracle stands in for the kernels),
the histograms are summed across ranks, and the result equals one process
running all devices -- the reference's multi-GPU histogram sum
(muca_delta_multigpu.cu:404-429)."""
import os
import socket

import numpy as np
import pytest


def test_shard_devices():
    from muca_gb300.shard import shard_devices
    assert [shard_devices(2, r, 5) for r in range(2)] == [(0, 3), (3, 2)]
    assert [shard_devices(4, r, 4) for r in range(4)] == [(0, 1), (1, 1), (2, 1), (3, 1)]
    seen = []
    for r in range(3):
        off, n = shard_devices(3, r, 8)
        seen += list(range(off, off + n))
    assert seen == list(range(8))
    with pytest.raises(ValueError):
        shard_devices(4, 0, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, L, cpd, ndev, out):
    import torch.distributed as dist
    from oracle import orc
    from muca_gb300.shard import shard_devices, reduce_histogram, max_over_ranks
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    N = L * L
    off, n = shard_devices(world, rank, ndev)
    h = np.zeros(N + 1, np.uint64)
    w32 = (np.cumsum(np.random.default_rng(1).normal(0, 1, N + 1)) * 0.5).astype(np.float32)
    for d in range(off, off + n):
        lat = orc.init_lattice(L, cpd, orc.scheme_weight(0, d))
        ej, ed, _ = orc.energies(L, lat)
        orc.weight_sweep(L, lat, ej, ed, w32, 3, 100 + 1000 * d, N, 3 * N, hist=h)
    tot = reduce_histogram(h)
    t = max_over_ranks(float(rank + 1))
    if rank == 0:
        np.save(out, tot)
        assert t == float(world)
    dist.destroy_process_group()


def test_two_rank_histogram_sum_equals_all_devices(tmp_path):
    import torch.multiprocessing as mp
    from oracle import orc
    orc.build()
    L, cpd, ndev = 8, 24, 3
    out = str(tmp_path / "h.npy")
    mp.spawn(_worker, args=(2, _free_port(), L, cpd, ndev, out), nprocs=2, join=True)
    tot = np.load(out)
    N = L * L
    h = np.zeros(N + 1, np.uint64)
    w32 = (np.cumsum(np.random.default_rng(1).normal(0, 1, N + 1)) * 0.5).astype(np.float32)
    for d in range(ndev):
        lat = orc.init_lattice(L, cpd, orc.scheme_weight(0, d))
        ej, ed, _ = orc.energies(L, lat)
        orc.weight_sweep(L, lat, ej, ed, w32, 3, 100 + 1000 * d, N, 3 * N, hist=h)
    np.testing.assert_array_equal(tot, h)
    assert int(tot.sum()) == ndev * cpd * 3 * N
