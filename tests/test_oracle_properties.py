"""Properties of the oracle's sweeps that hold whatever the random numbers
(the oracle restates the reference kernels mcs, muca_delta_multigpu.cu:737-829
and produce2_multigpu.cu:401-496, and is the checker of every GPU parity
test): the running energies E_J, E_Delta and M equal the lattice's after a
sweep, the histograms hold one entry per recorded attempt, the results do
not depend on the host thread count, and chain ranges are independent
(chain0 selects a chain's keys, so a range swept alone gives the same
chains as the whole set)."""
import numpy as np
import pytest


def _setup(orc, L, nch, produce, seed):
    N = L * L
    scheme = orc.scheme_produce(0) if produce else orc.scheme_weight(0, 0)
    lat = orc.init_lattice(L, nch, scheme).reshape(nch, N).copy()
    ej, ed, mg = orc.energies(L, lat)
    rng = np.random.default_rng(seed)
    w = np.cumsum(rng.normal(-0.2, 0.8, N + 1))
    return lat, ej.copy(), ed.copy(), mg.copy(), w


def _sweep(orc, L, produce, lat, ej, ed, mg, w, therm, nup, chain0=0, nthreads=1):
    lat = lat.copy()
    ej, ed, mg = ej.copy(), ed.copy(), mg.copy()
    if produce:
        lat, h = orc.produce_sweep(L, lat, ej, ed, mg, w, 3, 100, therm, nup, chain0=chain0, nthreads=nthreads)
    else:
        lat, h = orc.weight_sweep(L, lat, ej, ed, w.astype(np.float32), 3, 100, therm, nup, chain0=chain0,
                                  nthreads=nthreads)
    return lat, ej, ed, mg, h


@pytest.mark.parametrize("produce", [False, True])
@pytest.mark.parametrize("L", [8, 12])
def test_running_energies_and_histogram_totals(orc, L, produce):
    N = L * L
    nch = 6
    lat, ej, ed, mg, w = _setup(orc, L, nch, produce, L)
    therm, nup = N + 3, 2 * N + 5
    lat1, ej1, ed1, mg1, h = _sweep(orc, L, produce, lat, ej, ed, mg, w, therm, nup)
    rj, rd, rm = orc.energies(L, lat1)
    np.testing.assert_array_equal(ej1, rj)
    np.testing.assert_array_equal(ed1, rd)
    if produce:
        np.testing.assert_array_equal(mg1, rm)
    assert int(h.sum()) == nch * nup
    assert not np.array_equal(lat1, lat)  # the sweep moved
    # spins stay in {-1, 0, 1}
    assert set(np.unique(lat1)) <= {-1, 0, 1}


@pytest.mark.parametrize("produce", [False, True])
def test_results_do_not_depend_on_the_thread_count(orc, produce):
    L, nch = 8, 9
    N = L * L
    lat, ej, ed, mg, w = _setup(orc, L, nch, produce, 3)
    a = _sweep(orc, L, produce, lat, ej, ed, mg, w, N, 3 * N + 1, nthreads=1)
    b = _sweep(orc, L, produce, lat, ej, ed, mg, w, N, 3 * N + 1, nthreads=4)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("produce", [False, True])
def test_chain_ranges_are_independent(orc, produce):
    L, nch, cut = 8, 7, 3
    N = L * L
    lat, ej, ed, mg, w = _setup(orc, L, nch, produce, 5)
    whole = _sweep(orc, L, produce, lat, ej, ed, mg, w, N + 1, 2 * N)
    lo = _sweep(orc, L, produce, lat[:cut], ej[:cut], ed[:cut], mg[:cut], w, N + 1, 2 * N)
    hi = _sweep(orc, L, produce, lat[cut:], ej[cut:], ed[cut:], mg[cut:], w, N + 1, 2 * N, chain0=cut)
    for k in range(4):
        np.testing.assert_array_equal(whole[k], np.concatenate([lo[k], hi[k]]))
    np.testing.assert_array_equal(whole[4], lo[4] + hi[4])


def test_thermalisation_records_nothing(orc):
    L, nch = 8, 4
    N = L * L
    lat, ej, ed, mg, w = _setup(orc, L, nch, False, 9)
    lat1, ej1, ed1, _, h = _sweep(orc, L, False, lat, ej, ed, mg, w, 3 * N, 0)
    assert int(h.sum()) == 0
    assert not np.array_equal(lat1, lat)
    rj, rd, _ = orc.energies(L, lat1)
    np.testing.assert_array_equal(ej1, rj)
    np.testing.assert_array_equal(ed1, rd)


@pytest.mark.parametrize("program", ["muca_mag", "produce_cpu"])
def test_cpu_programs_keep_energies_and_counts(orc, program):
    """The CPU programs' sweeps restated in the oracle (muca_mag.cpp:312-393,
    random sites with three streams; produce.cpp mcs): one chain per worker,
    running E_J, E_Delta (and M) equal to the lattice's, one histogram entry
    per production attempt."""
    L = 10
    N = L * L
    Lb = orc.lib()
    rng = np.random.default_rng(11)
    w = np.cumsum(rng.normal(-0.2, 0.8, N + 1))
    therm, nup = 2 * N + 1, 3 * N + 7
    for worker in range(3):
        scheme = orc.scheme_muca_mag(0) if program == "muca_mag" else Lb.orc_scheme_produce_cpu(0)
        s = orc.init_lattice(L, 1, scheme, chain0=worker).reshape(-1).copy()
        ej, ed, mg = (np.array([v[0]], np.int32) for v in orc.energies(L, s[None, :]))
        if program == "muca_mag":
            h = np.zeros(N + 1, np.uint64)
            Lb.orc_muca_mag_mcs(L, worker, s, ej, ed, w, h, 2, 100, therm, nup)
        else:
            h = np.zeros((N + 1) * (N + 2) // 2, np.uint64)
            Lb.orc_produce_cpu_mcs(L, worker, s, ej, ed, mg, w, h, 0, 100, therm, nup)
        rj, rd, rm = orc.energies(L, s[None, :])
        assert (ej[0], ed[0]) == (rj[0], rd[0])
        if program == "produce_cpu":
            assert mg[0] == rm[0]
        assert int(h.sum()) == nup
        assert set(np.unique(s)) <= {-1, 0, 1}
