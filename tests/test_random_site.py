"""The random-site algorithm of the reference's CPU weight program
(muca_mag.cpp:312-393) and of its GPU port mcs2 (muca_delta_multigpu.cu:637-734)
on the device, against the oracle's restatement of muca_mag's mcs (itself
pinned against the reference source, tests/test_oracle.py): with the host
libm's logf (host_logf=1) the GPU reproduces the CPU program bit for bit;
with CUDA's logf it is mcs2."""
import ctypes

import numpy as np
import pytest


def test_random_site_rejects_bad_params():
    from muca_gb300 import build as b
    b.build()
    import muca_gb300 as m
    for kw in (dict(mode=m.MODE_PRODUCE), dict(ndev=2), dict(algorithm=2)):
        with pytest.raises(m.MucaError):
            m.Engine(16, nchains=32, algorithm=kw.pop("algorithm", m.ALGO_RANDOM_SITE), **kw)


def _oracle_chains(orc, L, nc, jack, lnw, it, seed, therm, nup, lat, ej, ed):
    N = L * L
    Lb = orc.lib()
    h = np.zeros(N + 1, np.uint64)
    hc = np.zeros(N + 1, np.uint64)
    for c in range(nc):
        s = np.ascontiguousarray(lat[c])
        e1 = np.array([ej[c]], np.int32)
        e2 = np.array([ed[c]], np.int32)
        Lb.orc_muca_mag_mcs(L, c, s, e1, e2, lnw, hc, it, seed, therm, nup)
        lat[c] = s
        ej[c], ed[c] = e1[0], e2[0]
        h += hc
    return lat, ej, ed, h


@pytest.mark.gpu
@pytest.mark.parametrize("host_logf", [1, 0])
@pytest.mark.parametrize("L,nc,therm,nup,weights,bracket", [
    (16, 4, 0, 5000, "walk", None), (12, 40, 300, 2000, "walk", None), (72, 64, 100, 3000, "walk", None),
    (72, 96, 0, 4000, "muca", None), (16, 40, 100, 3000, "walk", 1e30), (72, 64, 0, 2000, "muca", 1e30)])
def test_random_site_sweep_vs_oracle(muca, orc, host_logf, L, nc, therm, nup, weights, bracket):
    """Bit-exact with the oracle; the FP32 fast test decides most attempts and
    the reference's FP64 test the ones in its band.  bracket = 1e30 sends
    every attempt to the FP64 test (the exact path on its own).  "muca"
    weights have the drift of a converged multicanonical weight (range of
    lnW ~ 3000 at L = 72)."""
    N = L * L
    rng = np.random.default_rng(L + nup)
    if weights == "walk":
        lnw = np.cumsum(rng.normal(0.0, 1.5, N + 1)) * 0.5
    else:
        lnw = np.cumsum(rng.normal(-0.6, 0.3, N + 1))
        lnw -= lnw[0]
    jack, it = 1, 7
    if host_logf:
        orc.use_device_logf(False)  # the CPU program's logf is the host's
    with muca.Engine(L, nchains=nc, algorithm=muca.ALGO_RANDOM_SITE, host_logf=host_logf) as e:
        if bracket is not None:
            e.set_log_bracket(bracket)
        e.set_weights(lnw)
        e.init_chains(muca.INIT_MUCA_MAG, jack)
        lat0 = e.get_lattice()
        ej0, ed0, _ = e.chain_state()
        e.sweep(it, jack, 0, therm, nup)
        lat1 = e.get_lattice()
        ej1, ed1, _ = e.chain_state()
        h = e.histogram()
    exp0 = orc.init_lattice(L, nc, orc.scheme_muca_mag(jack))
    np.testing.assert_array_equal(lat0, exp0)
    ol, oj, od, oh = _oracle_chains(orc, L, nc, jack, lnw, it, jack, therm, nup, lat0.copy(),
                                    ej0.astype(np.int32).copy(), ed0.astype(np.int32).copy())
    np.testing.assert_array_equal(lat1, ol)
    np.testing.assert_array_equal(ej1, oj)
    np.testing.assert_array_equal(ed1, od)
    np.testing.assert_array_equal(h, oh)
    assert int(h.sum()) == nc * nup


@pytest.mark.gpu
@pytest.mark.parametrize("continuing", [0, 1])
def test_random_site_weight_run_vs_oracle(muca, orc, continuing):
    """The CPU program's whole loop (muca_mag.cpp:129-183): NUP*1.05 at the
    top of every iteration, mcs of every rank with therm 0, histogram sum,
    the CPU-flavour update (held until full width when continuing)."""
    L, nc, M, max_iter = 8, 4, 300, 40
    N = L * L
    orc.use_device_logf(False)
    with muca.Engine(L, nchains=nc, algorithm=muca.ALGO_RANDOM_SITE, host_logf=1) as e:
        res, recs = e.weight_run(starting_M=M, jack=0, rule=muca.UPDATE_TRIVIAL_CPU, hold_until_full=continuing,
                                 nup_schedule=4, max_iter=max_iter, init_scheme=muca.INIT_MUCA_MAG, records=max_iter)
        w = e.get_weights()
    o = orc.WeightOpts(L=L, nchains=nc, jack=0, gpu=0, starting_M=M, recursive=2, hold_until_full=continuing,
                       flat_minmean=0, max_iter=max_iter, rounds=7, nthreads=1, sched=4, algo=1)
    lat = orc.init_lattice(L, nc, orc.scheme_muca_mag(0)).reshape(-1).copy()
    ej, ed, _ = orc.energies(L, lat.reshape(nc, N))
    lnw = np.zeros(N + 1)
    pacc = np.zeros(N + 1)
    rec = np.zeros(5 * max_iter)
    conv = ctypes.c_int()
    it = orc.lib().orc_weight_run(ctypes.byref(o), lat, ej, ed, lnw, pacc, rec, max_iter, ctypes.byref(conv))
    assert (res.iterations, res.converged) == (it, conv.value)
    rec = rec.reshape(max_iter, 5)
    for k, r in enumerate(recs[:it]):
        assert r.nupdates == int(rec[k, 2]), k
        assert r.width_temp == int(rec[k, 0]), k
        assert r.total_run == int(rec[k, 3]), k
    np.testing.assert_allclose(w, lnw, rtol=1e-12, atol=1e-9)


def test_row_from_high_product_is_exact():
    """The random-site kernel forms row = idx / L as the high 32 bits of
    idx * ceil(2^32 / L); exact for every site index of every L in 3..128."""
    for L in range(3, 129):
        N = L * L
        inv = ((1 << 32) + L - 1) // L
        idx = np.arange(N, dtype=np.uint64)
        assert np.array_equal((idx * np.uint64(inv)) >> np.uint64(32), idx // np.uint64(L)), L
