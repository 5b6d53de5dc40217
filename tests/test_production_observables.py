"""Production with a converged weight, end to end, against the oracle and
against the reference's CPU production algorithm.

The L=128 production configuration at a size the oracle finishes in
seconds: a weight converged on the device (the trivial update to
min/mean >= 0.5), then the reference production loop with jackknife blocks
(thermalisation launch, then blocks with the seeds of
produce2_multigpu.cu:324-347; the JACKS blocks of produce.cpp:201-247),
each block's 2D (E_Delta, M) histogram reweighted at Delta = 1.96
(produce2_multigpu.cu:293-300,498-518).

1. With the same seeds the device's block histograms equal the oracle's bit
   for bit, and so the observables and their jackknife errors agree to
   1e-12.
2. The reference CPU program's algorithm (produce.cpp mcs: its own keys,
   double-precision uniforms, one chain per rank, restated in the oracle and
   pinned to the reference source) samples the same multicanonical
   distribution with independent random numbers; its jackknifed <|M|>, chi
   and U4 agree with the device's within the combined jackknife errors
   (3 sigma; with the fixed seeds here the test is deterministic).  Each of
   its blocks starts from
   a cleared histogram: produce.cpp clears only the first N+1 bins of its 2D
   histogram (:429), so its blocks are not independent as written.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L, BETA, DELTA = 16, 2.0, 1.96
N = L * L
CHAINS, THERM_SWEEPS, BLOCKS, BLOCK_SWEEPS = 256, 50, 10, 200


@pytest.fixture(scope="module")
def converged(muca):
    with muca.Engine(L, nchains=512) as e:
        res, _ = e.weight_run(starting_M=N, rule=muca.UPDATE_TRIVIAL, nup_schedule=1, flat_minmean=1, max_iter=5000,
                              nup_max=1 << 16, init_scheme=muca.INIT_CHAIN_COUNTER, records=1, graph_iters=16)
        w = e.get_weights()
    assert res.converged
    return w


def _obs_from_hist(orc, h, w):
    ws = w.copy()
    orc.lib().orc_weight_shift(BETA, DELTA, N, ws)
    bz = np.zeros(N + 1)
    orc.lib().orc_boltz(BETA, DELTA, N, ws, bz, 0)
    return orc.observables(BETA, N, h, bz)


@pytest.fixture(scope="module")
def device_run(muca, converged):
    w = converged
    blocks = []
    with muca.Engine(L, nchains=CHAINS, mode=muca.MODE_PRODUCE) as e:
        e.init_chains(muca.INIT_PRODUCE, 0)
        e.set_weights(w)
        e.weight_shift(BETA, DELTA)
        lat0 = e.get_lattice()
        st0 = e.chain_state()
        e.sweep(0, 100, 1000, THERM_SWEEPS * N, 0)
        for jj in range(BLOCKS):
            e.sweep(jj, 100, 2000, 0, BLOCK_SWEEPS * N)
            o = e.observables(BETA, DELTA)
            blocks.append((e.histogram(), (o.m_abs, o.chi, o.u4), (o.sum, o.m1, o.m2, o.m4)))
        jk = [e.jackknife(np.array([b[1][i] for b in blocks])) for i in range(3)]
    return lat0, st0, blocks, jk


def test_block_histograms_and_observables_vs_oracle(orc, converged, device_run):
    w = converged
    lat0, (ej0, ed0, mg0), blocks, jk = device_run
    lat = lat0.copy()
    ej, ed, mg = (np.ascontiguousarray(x, np.int32).copy() for x in (ej0, ed0, mg0))
    orc.produce_sweep(L, lat, ej, ed, mg, w, 0, 100, THERM_SWEEPS * N, 0, nthreads=8)
    per_block = []
    for jj, (h, ob, sums) in enumerate(blocks):
        _, oh = orc.produce_sweep(L, lat, ej, ed, mg, w, jj, 100, 0, BLOCK_SWEEPS * N, nthreads=8)
        assert np.array_equal(h, oh), "block %d histogram differs from the oracle" % jj
        o = _obs_from_hist(orc, oh, w)
        np.testing.assert_allclose(ob, o[:3], rtol=1e-12)
        np.testing.assert_allclose(sums, o[3:], rtol=1e-12)
        per_block.append(o[:3])
    per_block = np.array(per_block)
    for i in range(3):
        oa, oe = orc.jackknife(per_block[:, i])
        np.testing.assert_allclose(jk[i], (oa, oe), rtol=1e-10)


def test_observables_agree_with_the_cpu_program_within_jackknife_errors(orc, converged, device_run):
    from concurrent.futures import ThreadPoolExecutor
    w = converged
    _, _, _, jk = device_run
    Lb = orc.lib()
    ranks = 64
    hs = (N + 1) * (N + 2) // 2
    lats, states = [], []
    for r in range(ranks):
        lat = orc.init_lattice(L, 1, Lb.orc_scheme_produce_cpu(0), chain0=r).reshape(-1).copy()
        states.append(tuple(np.array([v[0]], np.int32) for v in orc.energies(L, lat[None, :])))
        lats.append(lat)

    def run(r, k, therm, nup):
        h = np.zeros(hs, np.uint64)
        ej, ed, mg = states[r]
        Lb.orc_produce_cpu_mcs(L, r, lats[r], ej, ed, mg, w, h, 0, k, therm, nup)
        return h

    per_block = []
    with ThreadPoolExecutor(16) as ex:
        # produce.cpp's thermalisation call: mcs(..., seed = SEED + 1000, therm_run, 0)
        list(ex.map(lambda r: run(r, 100 + 1000, THERM_SWEEPS * N, 0), range(ranks)))
        for k in range(BLOCKS):
            hsum = sum(ex.map(lambda r: run(r, k, 0, BLOCK_SWEEPS * N), range(ranks)))
            per_block.append(_obs_from_hist(orc, hsum, w)[:3])
    per_block = np.array(per_block)
    names = ("<|M|>", "chi", "U4")
    for i in range(3):
        ca, ce = orc.jackknife(per_block[:, i])
        ga, ge = jk[i]
        z = abs(ga - ca) / np.hypot(ge, ce)
        print("%s: device %.8g +- %.2g, CPU program %.8g +- %.2g: %.2f sigma" % (names[i], ga, ge, ca, ce, z))
        assert np.isfinite(z) and z < 3.0, "%s: device %.6g +- %.2g, CPU program %.6g +- %.2g (%.2f sigma)" % (
            names[i], ga, ge, ca, ce, z)
