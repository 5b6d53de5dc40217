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


class _OracleEngine:
    """The step API of muca_gb300.Engine on the oracle, for the reference
    devices `devs` (weight mode, the reference's initial spins of jack 0)."""

    def __init__(self, L, cpd, devs):
        from oracle import orc
        self.orc, self.L, self.N, self.devs = orc, L, L * L, list(devs)
        self.lat, self.ej, self.ed = {}, {}, {}
        for d in self.devs:
            self.lat[d] = orc.init_lattice(L, cpd, orc.scheme_weight(0, d)).copy()
            self.ej[d], self.ed[d], _ = orc.energies(L, self.lat[d])
        self.lnw = np.zeros(self.N + 1)
        self.h = np.zeros(self.N + 1, np.uint64)

    def sweep(self, k, seed_base, seed_dev_mul, therm, nup):
        w32 = self.lnw.astype(np.float32)  # the FP32 shadow of the weight kernel
        self.h[:] = 0
        for d in self.devs:
            self.orc.weight_sweep(self.L, self.lat[d], self.ej[d], self.ed[d], w32, k, seed_base + seed_dev_mul * d,
                                  therm, nup, hist=self.h)

    def histogram(self):
        return self.h.copy()

    def set_histogram(self, h):
        self.h[:] = h

    def hist_stats(self):
        from types import SimpleNamespace
        s, e = self.orc.hist_range(self.h)
        return SimpleNamespace(start=s, end=e, d_kl=self.orc.kull_leibler(self.h),
                               min_over_mean=self.orc.flatness(self.h))

    def update_weights(self, rule):
        assert rule == 0
        self.orc.lib().orc_update_trivial_gpu(self.h, self.N, self.lnw)


RUN = dict(starting_M=64, flat_minmean=1, max_iter=400, nup_schedule=1, nup_max=1 << 12)


def _run_worker(rank, world, port, L, cpd, ndev, out):
    import torch.distributed as dist
    from muca_gb300.shard import shard_devices, weight_run_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    off, n = shard_devices(world, rank, ndev)
    eng = _OracleEngine(L, cpd, range(off, off + n))
    res = weight_run_sharded(eng, ndev * cpd, **RUN)
    np.save(out % rank, np.concatenate([eng.lnw, [res["iterations"], res["converged"], res["total_run"]]]))
    dist.destroy_process_group()


def test_two_rank_weight_run_equals_one_process():
    """The multi-device weight loop over 2 gloo ranks (one reference device
    each, histograms summed every iteration) gives, on both ranks, the
    weights of one process that sweeps both devices."""
    import tempfile
    import torch.multiprocessing as mp
    from oracle import orc
    from muca_gb300.shard import weight_run_sharded
    orc.build()
    L, cpd, ndev = 8, 32, 2
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "r%d.npy")
        mp.spawn(_run_worker, args=(2, _free_port(), L, cpd, ndev, out), nprocs=2, join=True)
        r0, r1 = np.load(out % 0), np.load(out % 1)
    eng = _OracleEngine(L, cpd, range(ndev))
    res = weight_run_sharded(eng, ndev * cpd, **RUN)
    one = np.concatenate([eng.lnw, [res["iterations"], res["converged"], res["total_run"]]])
    assert res["converged"]
    np.testing.assert_array_equal(r0, one)
    np.testing.assert_array_equal(r1, one)


GPU_RUN = dict(starting_M=256, flat_minmean=1, max_iter=200, nup_schedule=1, nup_max=1 << 14)


@pytest.mark.gpu
def test_sharded_loop_equals_device_run(muca):
    """One process with both reference devices: the host-driven sharded loop
    reproduces the device-side run (muca_weight_run) bit for bit."""
    from muca_gb300.shard import weight_run_sharded
    L, cpd, ndev = 16, 128, 2
    with muca.Engine(L, nchains=cpd, ndev=ndev) as e:
        r, _ = e.weight_run(records=1, **GPU_RUN)
        w_dev = e.get_weights()
    with muca.Engine(L, nchains=cpd, ndev=ndev) as e:
        e.init_chains(muca.INIT_WEIGHT, 0)
        res = weight_run_sharded(e, cpd * ndev, **GPU_RUN)
        w_host = e.get_weights()
    assert r.converged and res["converged"]
    assert (res["iterations"], res["total_run"], res["width_reached_iter"]) == \
        (r.iterations, r.total_run, r.width_reached_iter)
    np.testing.assert_array_equal(w_host, w_dev)


def _gpu_worker(rank, world, port, L, cpd, out):
    import torch.distributed as dist
    import muca_gb300 as m
    from muca_gb300.shard import weight_run_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    with m.Engine(L, nchains=cpd, ndev=1, dev_offset=rank) as e:
        e.init_chains(m.INIT_WEIGHT, 0)
        res = weight_run_sharded(e, cpd * world, **GPU_RUN)
        np.save(out % rank, np.concatenate([e.get_weights(), [res["iterations"], res["total_run"]]]))
    dist.destroy_process_group()


@pytest.mark.gpu
def test_two_process_weight_run_equals_two_devices(muca, tmp_path):
    """Two processes, one reference device each, histograms summed over gloo
    every iteration (the kernels never wait on each other: the exchange is
    on the host): both end with the weights of one context running both
    devices."""
    import torch.multiprocessing as mp
    L, cpd = 16, 128
    out = str(tmp_path / "r%d.npy")
    mp.spawn(_gpu_worker, args=(2, _free_port(), L, cpd, out), nprocs=2, join=True)
    with muca.Engine(L, nchains=cpd, ndev=2) as e:
        r, _ = e.weight_run(records=1, **GPU_RUN)
        ref = np.concatenate([e.get_weights(), [r.iterations, r.total_run]])
    for k in range(2):
        np.testing.assert_array_equal(np.load(out % k), ref)
