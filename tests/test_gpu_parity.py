"""GPU parity: the sm_103a kernels against the CPU oracle and against the
reference's own kernels (muca_delta_multigpu.cu / produce2_multigpu.cu
compiled unchanged into cubins and launched through oracle/refgpu.cpp).

Integer results (lattices, E_J, E_Delta, M, histograms) must be bit-exact;
FP64 weights within 1e-12 relative (1e-9 absolute near zero); observables
within 1e-12 relative.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 100


def _weights(N, rng, sigma=1.5):
    # a log-weight whose differences straddle the Metropolis threshold
    return np.cumsum(rng.normal(0.0, sigma, N + 1)) * 0.5


def _oracle_weight_sweep(orc, L, lat, ej, ed, w32, it, therm, nup, ndev, cpd, rounds=7):
    """the oracle over `ndev` emulated devices of `cpd` chains each"""
    N = L * L
    lat = lat.copy()
    ej = ej.copy()
    ed = ed.copy()
    h = np.zeros(N + 1, np.uint64)
    for d in range(ndev):
        sl = slice(d * cpd, (d + 1) * cpd)
        sub, _ = orc.weight_sweep(L, lat[sl], ej[sl], ed[sl], w32, it, SEED + 1000 * d, therm, nup,
                                  chain0=0, rounds=rounds, nthreads=8, hist=h)
        lat[sl] = sub
    return lat, ej, ed, h


def _ej_ed_copy(a):
    return np.ascontiguousarray(a, np.int32).copy()


def _kernels(L):
    """sweep kernels applicable to L: generic always, windowed and
    warp-specialised when L % 8 == 0"""
    return [1, 2, 3] if (L % 8 == 0 and L >= 8) else [1]


def _with_kernels(cases):
    return [c + (k,) for c in cases for k in _kernels(c[0])]


@pytest.mark.parametrize("L,cpd,ndev,jack", [(4, 256, 1, 0), (6, 100, 2, 1), (8, 256, 1, 3), (16, 300, 2, 0),
                                             (72, 64, 1, 2), (10, 33, 3, 0)])
def test_init_weight_scheme(muca, orc, L, cpd, ndev, jack):
    with muca.Engine(L, nchains=cpd, ndev=ndev) as e:
        e.init_chains(muca.INIT_WEIGHT, jack)
        lat = e.get_lattice()
        ej, ed, mg = e.chain_state()
    exp = np.concatenate([orc.init_lattice(L, cpd, orc.scheme_weight(jack, d)) for d in range(ndev)])
    np.testing.assert_array_equal(lat, exp)
    oj, od, om = orc.energies(L, exp)
    np.testing.assert_array_equal(ej, oj)
    np.testing.assert_array_equal(ed, od)
    np.testing.assert_array_equal(mg, om)


@pytest.mark.parametrize("L,cpd,ndev", [(4, 256, 2), (16, 100, 1), (24, 64, 1)])
def test_init_produce_scheme(muca, orc, L, cpd, ndev):
    with muca.Engine(L, nchains=cpd, ndev=ndev, mode=muca.MODE_PRODUCE) as e:
        e.init_chains(muca.INIT_PRODUCE, 0)
        lat = e.get_lattice()
    exp = np.concatenate([orc.init_lattice(L, cpd, orc.scheme_produce(d)) for d in range(ndev)])
    np.testing.assert_array_equal(lat, exp)


@pytest.mark.parametrize("L,cpd,ndev,jack", [(16, 256, 2, 0), (24, 100, 1, 3), (72, 64, 1, 0)])
def test_init_graded_scheme(muca, orc, L, cpd, ndev, jack):
    """MUCA_INIT_GRADED: the weight scheme's Philox words, worker W's spins
    nonzero with probability (2W+1)/(2 cpd); E_Delta spreads over [0, N]."""
    with muca.Engine(L, nchains=cpd, ndev=ndev) as e:
        e.init_chains(muca.INIT_GRADED, jack)
        lat = e.get_lattice()
        ej, ed, mg = e.chain_state()
    exp = np.concatenate([orc.init_lattice_graded(L, cpd, orc.scheme_weight(jack, d), cpd) for d in range(ndev)])
    np.testing.assert_array_equal(lat, exp)
    oj, od, om = orc.energies(L, exp)
    np.testing.assert_array_equal(ej, oj)
    np.testing.assert_array_equal(ed, od)
    N = L * L
    frac = od[:cpd] / N
    target = (np.arange(cpd) + 0.5) / cpd
    assert np.abs(frac - target).max() < 5.0 / np.sqrt(N)


def test_set_get_lattice_roundtrip(muca, orc):
    rng = np.random.default_rng(5)
    for L in (3, 16, 72):
        with muca.Engine(L, nchains=70) as e:
            lat = rng.integers(-1, 2, (70, L * L)).astype(np.int8)
            e.set_lattice(lat)
            np.testing.assert_array_equal(e.get_lattice(), lat)
            oj, od, om = orc.energies(L, lat)
            ej, ed, mg = e.chain_state()
            np.testing.assert_array_equal(ej, oj)
            np.testing.assert_array_equal(ed, od)
            np.testing.assert_array_equal(mg, om)
            bad = lat.copy()
            bad[3, 5] = 2
            with pytest.raises(muca.MucaError):
                e.set_lattice(bad)


# (L, chains per device, emulated devices, therm, nup): fast kernel for L % 8 == 0,
# generic kernel otherwise; partial windows, sweep wrap-around, therm only, nup only
SWEEPS = [
    (8, 256, 1, 64, 1), (8, 256, 1, 64, 13), (16, 200, 2, 256, 1000), (24, 96, 1, 0, 3 * 576 + 5),
    (72, 64, 1, 5184, 37), (72, 40, 2, 100, 5184 + 9), (32, 128, 1, 1024, 0),
    (4, 256, 1, 16, 333), (6, 100, 2, 36, 77), (10, 64, 1, 100, 250), (2, 40, 1, 4, 50), (3, 32, 1, 9, 41),
]


@pytest.mark.parametrize("L,cpd,ndev,therm,nup,kernel", _with_kernels(SWEEPS))
def test_weight_sweep_vs_oracle(muca, orc, L, cpd, ndev, therm, nup, kernel):
    rng = np.random.default_rng(L * 1000 + nup)
    N = L * L
    lnw = _weights(N, rng)
    it = int(rng.integers(0, 50))
    with muca.Engine(L, nchains=cpd, ndev=ndev, kernel=kernel) as e:
        assert e.info.kernel == kernel
        e.set_weights(lnw)
        e.init_chains(muca.INIT_WEIGHT, 1)
        lat0 = e.get_lattice()
        ej0, ed0, _ = e.chain_state()
        e.sweep(it, SEED, 1000, therm, nup)
        lat1 = e.get_lattice()
        ej1, ed1, _ = e.chain_state()
        h = e.histogram()
    olat, oej, oed, oh = _oracle_weight_sweep(orc, L, lat0, _ej_ed_copy(ej0), _ej_ed_copy(ed0),
                                              lnw.astype(np.float32), it, therm, nup, ndev, cpd)
    np.testing.assert_array_equal(lat1, olat)
    np.testing.assert_array_equal(ed1, oed)
    np.testing.assert_array_equal(ej1, oej)
    np.testing.assert_array_equal(h, oh)
    assert int(h.sum()) == cpd * ndev * nup


@pytest.mark.parametrize("L,therm,nup,kernel", _with_kernels([(8, 64, 500), (16, 256, 300), (24, 576, 100),
                                                                (72, 5184, 41), (4, 16, 200), (6, 36, 99),
                                                                (10, 100, 57)]))
def test_weight_sweep_vs_reference_kernel(muca, orc, refgpu, L, therm, nup, kernel):
    rng = np.random.default_rng(L + 7)
    N = L * L
    lnw = _weights(N, rng)
    w32 = lnw.astype(np.float32)
    it = 3
    with muca.Engine(L, nchains=256, kernel=kernel) as e:
        e.set_weights(lnw)
        e.init_chains(muca.INIT_WEIGHT, 0)
        lat0 = e.get_lattice()
        ej0, ed0, _ = e.chain_state()
        e.sweep(it, SEED, 1000, therm, nup)
        lat1 = e.get_lattice()
        ej1, ed1, _ = e.chain_state()
        h = e.histogram()
    rl, rh, rej, red, _ = orc.refgpu_weight(L, lat0, w32, ej0, ed0, it, SEED, therm, nup)
    np.testing.assert_array_equal(lat1, rl)
    np.testing.assert_array_equal(ed1, red)
    np.testing.assert_array_equal(ej1, rej)
    np.testing.assert_array_equal(h, rh)


def test_reference_kernel_init_energies(muca, orc, refgpu):
    """computeEnergies/computeDeltaE of the reference against ours."""
    L = 16
    with muca.Engine(L, nchains=256) as e:
        e.init_chains(muca.INIT_WEIGHT, 0)
        lat0 = e.get_lattice()
        ej0, ed0, _ = e.chain_state()
    w32 = np.zeros(L * L + 1, np.float32)
    _, _, rej, red, _ = orc.refgpu_weight(L, lat0, w32, ej0 * 0, ed0 * 0, 0, SEED, 0, 0, compute_energies=True)
    np.testing.assert_array_equal(rej, ej0)
    np.testing.assert_array_equal(red, ed0)


@pytest.mark.parametrize("rounds", [7, 10])
@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_weight_sweep_rounds(muca, orc, rounds, kernel):
    L, cpd = 16, 96
    rng = np.random.default_rng(rounds)
    lnw = _weights(L * L, rng)
    with muca.Engine(L, nchains=cpd, rounds=rounds, kernel=kernel) as e:
        e.set_weights(lnw)
        e.init_chains(muca.INIT_WEIGHT, 0)
        lat0 = e.get_lattice()
        ej0, ed0, _ = e.chain_state()
        e.sweep(1, SEED, 1000, 256, 700)
        lat1 = e.get_lattice()
        h = e.histogram()
    olat, _, _, oh = _oracle_weight_sweep(orc, L, lat0, _ej_ed_copy(ej0), _ej_ed_copy(ed0), lnw.astype(np.float32),
                                          1, 256, 700, 1, cpd, rounds=rounds)
    np.testing.assert_array_equal(lat1, olat)
    np.testing.assert_array_equal(h, oh)


@pytest.mark.parametrize("L,cpd,therm,nup,kernel", _with_kernels([(8, 256, 64, 300), (16, 200, 0, 1000),
                                                                    (4, 100, 16, 123), (24, 64, 576, 50),
                                                                    (6, 64, 0, 200), (72, 40, 5184, 1000)]))
def test_produce_sweep_vs_oracle(muca, orc, L, cpd, therm, nup, kernel):
    rng = np.random.default_rng(L * 7 + nup)
    N = L * L
    lnw = _weights(N, rng)
    with muca.Engine(L, nchains=cpd, mode=muca.MODE_PRODUCE, kernel=kernel) as e:
        e.set_weights(lnw)
        e.init_chains(muca.INIT_PRODUCE, 0)
        lat0 = e.get_lattice()
        ej0, ed0, mg0 = e.chain_state()
        e.sweep(5, SEED, 2000, therm, nup)
        lat1 = e.get_lattice()
        ej1, ed1, mg1 = e.chain_state()
        h = e.histogram()
    a = lat0.copy()
    oej, oed, omg = _ej_ed_copy(ej0), _ej_ed_copy(ed0), _ej_ed_copy(mg0)
    olat, oh = orc.produce_sweep(L, a, oej, oed, omg, lnw, 5, SEED, therm, nup, nthreads=8)
    np.testing.assert_array_equal(lat1, olat)
    np.testing.assert_array_equal(ed1, oed)
    np.testing.assert_array_equal(ej1, oej)
    np.testing.assert_array_equal(mg1, omg)
    np.testing.assert_array_equal(h, oh)


@pytest.mark.parametrize("L,cpd,therm,nup", [(16, 128, 256, 700), (24, 64, 0, 1000), (72, 40, 100, 5184 + 9)])
@pytest.mark.parametrize("kernel", [2, 3])
@pytest.mark.parametrize("mode", ["weight", "produce"])
def test_exact_replay_alone_vs_oracle(muca, orc, L, cpd, therm, nup, kernel, mode):
    """With the fast test's bound at 1e30 every window of the windowed and
    warp-specialised kernels takes the exact replay (CUDA's logf; in
    production also the FP64 difference from the global weights): the
    oracle's lattices, energies and histograms all the same.  A bound below
    the measured one is refused."""
    rng = np.random.default_rng(L * 11 + nup + kernel)
    N = L * L
    lnw = _weights(N, rng)
    produce = mode == "produce"
    with muca.Engine(L, nchains=cpd, kernel=kernel, mode=muca.MODE_PRODUCE if produce else muca.MODE_WEIGHT) as e:
        measured = e.info.log_bracket
        assert 0.0 < measured < 1e-2
        with pytest.raises(muca.MucaError):
            e.set_log_bracket(measured * 0.5)
        with pytest.raises(muca.MucaError):
            e.set_log_bracket(float("nan"))
        e.set_log_bracket(1e30)
        e.set_weights(lnw)
        e.init_chains(muca.INIT_PRODUCE if produce else muca.INIT_WEIGHT, 0)
        lat0 = e.get_lattice()
        ej0, ed0, mg0 = e.chain_state()
        e.sweep(3, SEED, 2000 if produce else 1000, therm, nup)
        lat1 = e.get_lattice()
        ej1, ed1, mg1 = e.chain_state()
        h = e.histogram()
    if produce:
        oej, oed, omg = _ej_ed_copy(ej0), _ej_ed_copy(ed0), _ej_ed_copy(mg0)
        olat, oh = orc.produce_sweep(L, lat0.copy(), oej, oed, omg, lnw, 3, SEED, therm, nup, nthreads=8)
        np.testing.assert_array_equal(mg1, omg)
    else:
        olat, oej, oed, oh = _oracle_weight_sweep(orc, L, lat0, _ej_ed_copy(ej0), _ej_ed_copy(ed0),
                                                  lnw.astype(np.float32), 3, therm, nup, 1, cpd)
    np.testing.assert_array_equal(lat1, olat)
    np.testing.assert_array_equal(ed1, oed)
    np.testing.assert_array_equal(ej1, oej)
    np.testing.assert_array_equal(h, oh)


@pytest.mark.parametrize("L,therm,nup,kernel", _with_kernels([(8, 64, 300), (16, 256, 200), (4, 0, 150),
                                                                (6, 36, 100)]))
def test_produce_sweep_vs_reference_kernel(muca, orc, refgpu, L, therm, nup, kernel):
    rng = np.random.default_rng(L * 3 + 1)
    N = L * L
    lnw = _weights(N, rng)
    with muca.Engine(L, nchains=256, mode=muca.MODE_PRODUCE, kernel=kernel) as e:
        e.set_weights(lnw)
        e.init_chains(muca.INIT_PRODUCE, 0)
        lat0 = e.get_lattice()
        ej0, ed0, mg0 = e.chain_state()
        e.sweep(2, SEED, 2000, therm, nup)
        lat1 = e.get_lattice()
        ej1, ed1, mg1 = e.chain_state()
        h = e.histogram()
    rl, rh, rej, red, rmg, _ = orc.refgpu_produce(L, lat0, lnw, ej0, ed0, mg0, 2, SEED, therm, nup)
    np.testing.assert_array_equal(lat1, rl)
    np.testing.assert_array_equal(ed1, red)
    np.testing.assert_array_equal(ej1, rej)
    np.testing.assert_array_equal(mg1, rmg)
    np.testing.assert_array_equal(h, rh)


def test_sweep_accumulate_and_determinism(muca):
    L = 16
    outs = []
    for _ in range(2):
        with muca.Engine(L, nchains=128) as e:
            e.init_chains(muca.INIT_WEIGHT, 0)
            e.sweep(0, SEED, 1000, 256, 100)
            h1 = e.histogram()
            e.sweep(1, SEED, 1000, 0, 50, accumulate=True)
            h2 = e.histogram()
            outs.append((h1, h2, e.get_lattice()))
    assert int(outs[0][0].sum()) == 128 * 100 and int(outs[0][1].sum()) == 128 * 150
    for a, b in zip(outs[0], outs[1]):
        np.testing.assert_array_equal(a, b)


# ---- FP64 weight math on the device --------------------------------------------------------

def _rand_hist(rng, N, zeros=0.2):
    h = rng.integers(0, 5000, N + 1).astype(np.uint64)
    h[rng.random(N + 1) < zeros] = 0
    h[: 2] = [0, 1]
    return h


@pytest.mark.parametrize("N", [16, 64, 5184, 16384])
def test_hist_stats_vs_oracle(muca, orc, N):
    L = int(round(N ** 0.5))
    rng = np.random.default_rng(N)
    h = _rand_hist(rng, N)
    with muca.Engine(L, nchains=32) as e:
        e.set_histogram(h)
        s = e.hist_stats()
    assert (s.start, s.end) == orc.hist_range(h)
    assert s.width == s.end - s.start
    assert s.visited == int((h > 0).sum()) and s.events == int(h.sum()) and s.min_count == int(h.min())
    np.testing.assert_allclose(s.d_kl, orc.kull_leibler(h), rtol=1e-12)
    np.testing.assert_allclose(s.min_over_mean, orc.flatness(h), rtol=1e-14)


@pytest.mark.parametrize("rule", [0, 1, 2])
@pytest.mark.parametrize("N", [64, 5184])
def test_weight_update_vs_oracle(muca, orc, rule, N):
    L = int(round(N ** 0.5))
    rng = np.random.default_rng(N + rule)
    Lb = orc.lib()
    with muca.Engine(L, nchains=32) as e:
        lnw = rng.normal(0, 10, N + 1)
        pacc = np.zeros(N + 1)
        e.set_weights(lnw)
        ref = lnw.copy()
        for step in range(3):  # p_acc persists across updates
            h = _rand_hist(rng, N, zeros=0.05 if step else 0.3)
            e.set_histogram(h)
            e.update_weights(rule)
            if rule == 0:
                Lb.orc_update_trivial_gpu(h, N, ref)
            elif rule == 1:
                Lb.orc_update_trivial_cpu(h, N, ref)
            else:
                s, en = orc.hist_range(h)
                Lb.orc_weight_recursion(h, N, pacc, s, en, ref)
                ref -= ref[0]
            got = e.get_weights()
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("rule,hold,flat,sched", [(0, 0, 0, 0), (2, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, 0),
                                                   (1, 0, 0, 0), (0, 0, 1, 1), (2, 0, 1, 2), (0, 0, 1, 2),
                                                   (0, 0, 1, 3), (0, 0, 1, 5), (0, 0, 0, 5)])
def test_weight_run_vs_oracle(muca, orc, rule, hold, flat, sched):
    """Whole reference iteration loop (schedule, width, D_KL, update) on the
    device against orc_weight_run, iteration by iteration; sched 1, 2 and 3
    are the doubling schedules (once at full width / every iteration / once
    every bin is covered)."""
    # doubling every iteration: few iterations, so the oracle stays quick
    L, cpd, max_iter = 8, 256, (14 if sched == 2 else 60)
    nup_max = 3000 if sched in (1, 3, 5) else 0
    M = 64 if sched in (1, 3, 5) else 1  # reaches full width, then grows up to the cap
    N = L * L
    with muca.Engine(L, nchains=cpd) as e:
        res, recs = e.weight_run(starting_M=M, jack=0, rule=rule, hold_until_full=hold, flat_minmean=flat,
                                 max_iter=max_iter, nup_schedule=sched, nup_max=nup_max, records=max_iter)
        lat = e.get_lattice()
        w = e.get_weights()
    if rule == 1:
        pytest.skip("the CPU-flavour update has no oracle run loop; covered by test_weight_update_vs_oracle")
    o = orc.WeightOpts(L=L, nchains=cpd, jack=0, gpu=0, starting_M=M, recursive=1 if rule == 2 else 0,
                       hold_until_full=hold, flat_minmean=flat, max_iter=max_iter, rounds=7, nthreads=8, sched=sched,
                       nup_max=nup_max)
    olat = orc.init_lattice(L, cpd, orc.scheme_weight(0, 0)).reshape(-1).copy()
    oej, oed, _ = orc.energies(L, olat.reshape(cpd, N))
    lnw = np.zeros(N + 1)
    pacc = np.zeros(N + 1)
    rec = np.zeros(5 * max_iter)
    conv = ctypes.c_int()
    it = orc.lib().orc_weight_run(ctypes.byref(o), olat, oej, oed, lnw, pacc, rec, max_iter, ctypes.byref(conv))
    assert res.iterations == it
    assert res.converged == conv.value
    rec = rec.reshape(max_iter, 5)
    for k, r in enumerate(recs):
        assert r.width_temp == int(rec[k, 0]), k
        assert r.nupdates == int(rec[k, 2]), k
        assert r.total_run == int(rec[k, 3]), k
        np.testing.assert_allclose(r.d_kl, rec[k, 1], rtol=1e-10, atol=1e-15)
        np.testing.assert_allclose(r.min_over_mean, rec[k, 4], rtol=1e-12)
    np.testing.assert_array_equal(lat, olat.reshape(cpd, N))
    np.testing.assert_allclose(w, lnw, rtol=1e-12, atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("L", [4, 8])
def test_weight_run_later_jack_vs_oracle(muca, orc, L):
    """A second jack as the reference's jack loop runs it (muca_delta_multigpu.cu:336-382):
    fresh chains with key 10W + 2*mm, NUPDATES back at starting_M, the weights
    and the running width of the previous jack kept -- so the schedule grows
    NUPDATES before the first sweep."""
    cpd, max_iter = 256, 3000
    N = L * L
    o = orc.WeightOpts(L=L, nchains=cpd, jack=0, gpu=0, starting_M=1, recursive=0, hold_until_full=0,
                       flat_minmean=0, max_iter=max_iter, rounds=7, nthreads=8, width_start=0)
    lnw = np.zeros(N + 1)
    pacc = np.zeros(N + 1)
    rec = np.zeros(5 * max_iter)
    conv = ctypes.c_int()
    with muca.Engine(L, nchains=cpd) as e:
        r0, _ = e.weight_run(starting_M=1, jack=0, max_iter=max_iter, records=1)
        olat = orc.init_lattice(L, cpd, orc.scheme_weight(0, 0)).reshape(-1).copy()
        oej, oed, _ = orc.energies(L, olat.reshape(cpd, N))
        it0 = orc.lib().orc_weight_run(ctypes.byref(o), olat, oej, oed, lnw, pacc, rec, max_iter,
                                       ctypes.byref(conv))
        assert conv.value == 1 and r0.converged == 1 and r0.iterations == it0
        np.testing.assert_allclose(e.get_weights(), lnw, rtol=1e-12, atol=1e-9)
        res, recs = e.weight_run(starting_M=1, jack=1, max_iter=max_iter, width_start=N, records=max_iter)
        lat = e.get_lattice()
        w = e.get_weights()
    o.jack = 1
    o.width_start = N
    olat = orc.init_lattice(L, cpd, orc.scheme_weight(1, 0)).reshape(-1).copy()
    oej, oed, _ = orc.energies(L, olat.reshape(cpd, N))
    rec[:] = 0
    it = orc.lib().orc_weight_run(ctypes.byref(o), olat, oej, oed, lnw, pacc, rec, max_iter, ctypes.byref(conv))
    rec = rec.reshape(max_iter, 5)
    for k, r in enumerate(recs[:it]):
        assert r.nupdates == int(rec[k, 2]), k
        assert r.total_run == int(rec[k, 3]), k
        assert r.width_temp == int(rec[k, 0]), k
        np.testing.assert_allclose(r.d_kl, rec[k, 1], rtol=1e-10, atol=1e-15, err_msg="iteration %d" % k)
    assert res.iterations == it and res.converged == conv.value
    np.testing.assert_array_equal(lat, olat.reshape(cpd, N))
    np.testing.assert_allclose(w, lnw, rtol=1e-12, atol=1e-9)


# ---- production reweighting ----------------------------------------------------------------

@pytest.mark.parametrize("L,delta", [(4, 1.96), (8, 1.5), (16, 1.99)])
def test_observables_vs_oracle(muca, orc, L, delta):
    N = L * L
    beta = 2.0
    rng = np.random.default_rng(L)
    hs = (N + 1) * (N + 2) // 2
    h = rng.integers(0, 10000, hs).astype(np.uint64)
    h[rng.random(hs) < 0.4] = 0
    lnw = np.cumsum(rng.normal(-1.0, 0.5, N + 1))
    with muca.Engine(L, nchains=64, mode=muca.MODE_PRODUCE) as e:
        e.set_weights(lnw)
        e.set_histogram(h)
        e.weight_shift(beta, delta)
        shifted = e.reweighting_weights()
        np.testing.assert_array_equal(e.get_weights(), lnw)  # the sweep keeps the weights as set
        ob = e.observables(beta, delta)
    ref = lnw.copy()
    orc.lib().orc_weight_shift(beta, delta, N, ref)
    np.testing.assert_array_equal(shifted, ref)
    bz = np.zeros(N + 1)
    orc.lib().orc_boltz(beta, delta, N, ref, bz, 0)
    o = orc.observables(beta, N, h, bz)
    np.testing.assert_allclose([ob.m_abs, ob.chi, ob.u4], o[:3], rtol=1e-12)
    np.testing.assert_allclose([ob.sum, ob.m1, ob.m2, ob.m4], o[3:], rtol=1e-12)


def test_jackknife_vs_oracle(muca, orc):
    rng = np.random.default_rng(1)
    with muca.Engine(8, nchains=32) as e:
        for J in (1, 2, 5, 10, 37):
            x = rng.normal(2.0, 0.3, J)
            a, s = e.jackknife(x)
            oa, os_ = orc.jackknife(x)
            np.testing.assert_allclose(a, oa, rtol=1e-15)
            if J == 1:
                assert np.isnan(s) and np.isnan(os_)
            else:
                np.testing.assert_allclose(s, os_, rtol=1e-13)


# ---- full-size workload (L=72, 16384 chains) -------------------------------------------------

@pytest.mark.parametrize("kernel", [2, 3])
def test_full_size_L72_properties(muca, orc, kernel):
    """The benchmark workload: every chain's final E_Delta / E_J is
    consistent with its lattice, the histogram holds exactly chains*nup
    entries, and a subset of chains matches the oracle bit for bit."""
    L, nch = 72, 16384
    N = L * L
    rng = np.random.default_rng(72)
    lnw = _weights(N, rng, sigma=0.8)
    with muca.Engine(L, nchains=nch, kernel=kernel) as e:
        assert e.info.lattice_in_smem == 1 and e.info.kernel == kernel
        e.set_weights(lnw)
        e.init_chains(muca.INIT_WEIGHT, 0)
        lat0 = e.get_lattice()
        ej0, ed0, _ = e.chain_state()
        e.sweep(7, SEED, 1000, N, 2 * N + 8)
        lat1 = e.get_lattice()
        ej1, ed1, mg1 = e.chain_state()
        h = e.histogram()
    assert int(h.sum()) == nch * (2 * N + 8)
    oj, od, om = orc.energies(L, lat1)
    np.testing.assert_array_equal(ej1, oj)
    np.testing.assert_array_equal(ed1, od)
    for lo, hi in ((0, 48), (8190, 8200), (nch - 40, nch)):
        a = lat0[lo:hi].copy()
        ej, ed = _ej_ed_copy(ej0[lo:hi]), _ej_ed_copy(ed0[lo:hi])
        orc.weight_sweep(L, a, ej, ed, lnw.astype(np.float32), 7, SEED, N, 2 * N + 8, chain0=lo, nthreads=8)
        np.testing.assert_array_equal(lat1[lo:hi], a.reshape(hi - lo, N))
        np.testing.assert_array_equal(ed1[lo:hi], ed)


@pytest.mark.gpu
@pytest.mark.parametrize("rule", [0, 2])
def test_iterate_host_equals_separate_calls(muca, rule):
    """muca_iterate_host (weights in, sweep, update, weights and histogram out,
    one synchronisation) gives what the five separate calls give."""
    L, nc = 16, 256
    N = L * L
    rng = np.random.default_rng(3)
    w0 = np.cumsum(rng.normal(-0.5, 0.3, N + 1))
    w0 -= w0[0]
    runs = []
    for fused in (False, True):
        out = []
        with muca.Engine(L, nchains=nc) as e:
            e.init_chains(muca.INIT_WEIGHT, 0)
            w = w0.copy()
            for k in range(3):
                if fused:
                    wo, ho = np.zeros(N + 1), np.zeros(N + 1, np.uint64)
                    s = e.iterate_host(w, k, 100, 1000, N, 2 * N, rule, lnw_out=wo, hist_out=ho, stats=True)
                else:
                    e.set_weights(w)
                    e.sweep(k, 100, 1000, N, 2 * N)
                    s = e.update_weights(rule)
                    wo, ho = e.get_weights(), e.histogram()
                out.append((wo.copy(), ho.copy(), (s.start, s.end, s.width, s.events, s.d_kl)))
                w = wo
        runs.append(out)
    for (wa, ha, sa), (wb, hb, sb) in zip(*runs):
        np.testing.assert_array_equal(wa, wb)
        np.testing.assert_array_equal(ha, hb)
        assert sa == sb


@pytest.mark.parametrize("sched,graph_iters", [(0, 7), (1, 16), (4, 3)])
def test_weight_run_graph_equals_per_iteration(muca, sched, graph_iters):
    """graph_iters K: K iterations per CUDA-graph replay give the per-iteration
    loop's run: iterations, NUPDATES totals, weights, histogram, records."""
    L, nc = 16, 256
    kw = dict(starting_M=1, nup_schedule=sched, flat_minmean=1, max_iter=300, nup_max=1 << 14, records=400)
    out = []
    for g in (0, graph_iters):
        with muca.Engine(L, nchains=nc) as e:
            r, recs = e.weight_run(graph_iters=g, **kw)
            out.append((r, recs, e.get_weights(), e.histogram()))
    (ra, reca, wa, ha), (rb, recb, wb, hb) = out
    assert (ra.iterations, ra.converged, ra.total_run, ra.width_reached_iter) == \
        (rb.iterations, rb.converged, rb.total_run, rb.width_reached_iter)
    np.testing.assert_array_equal(wa, wb)
    np.testing.assert_array_equal(ha, hb)
    assert [(x.k, x.width, x.nupdates, x.total_run, x.d_kl) for x in reca] == \
        [(x.k, x.width, x.nupdates, x.total_run, x.d_kl) for x in recb]


def test_iterate_host_rejects_bad_calls(muca):
    L = 8
    N = L * L
    with muca.Engine(L, nchains=64) as e:
        w = np.zeros(N + 1)
        with pytest.raises(muca.MucaError, match="rule"):
            e.iterate_host(w, 0, 100, 1000, N, N, rule=7)
        w[3] = np.nan
        with pytest.raises(muca.MucaError, match="finite"):
            e.iterate_host(w, 0, 100, 1000, N, N)
        with pytest.raises(ValueError):
            e.iterate_host(np.zeros(N), 0, 100, 1000, N, N)
        # NULL in and out: the device weights are kept, nothing is copied
        e.iterate_host(None, 0, 100, 1000, N, N)
    with muca.Engine(L, nchains=64, mode=muca.MODE_PRODUCE) as e:
        with pytest.raises(muca.MucaError, match="weight-mode"):
            e.iterate_host(None, 0, 100, 1000, N, N)
