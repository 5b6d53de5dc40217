"""The CPU oracle pinned against the reference's own known answers.

* Philox4x32-7/-10 against Random123/examples/kat_vectors:24-29.
* u01fixedpt<float|double> against Random123/examples/ut_uniform_kat_vectors.dat.
* produce.cpp mcs and muca_mag.cpp mcs against outputs of those routines
  compiled from the reference sources (tests/golden/ref_cpu.npz).
* hist_range / kull_leibler / weight_recursion / jakknife / weight_shift /
  observables against the reference GPU programs' host routines
  (tests/golden/ref_hostmath.npz).
* the whole reference produce_mpi program (one rank) against a restatement
  of its main loop built from oracle routines (tests/golden/ref_produce_main.json).
Where the reference harness itself is present (oracle/_ref), the same
comparisons also run on fresh random inputs.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_philox_kat(orc):
    rows = json.load(open(os.path.join(GOLD, "philox_kat.json")))["rows"]
    assert len(rows) == 6
    for r in rows:
        out = orc.philox(r["ctr"], r["key"], r["rounds"])
        assert list(map(int, out)) == r["out"], r


def test_u01fixedpt_kat(orc):
    rows = json.load(open(os.path.join(GOLD, "u01_kat.json")))["rows"]
    assert len(rows) > 50
    L = orc.lib()
    for r in rows:
        exp = float(r["value"])
        if r["type"] == "float":
            got = L.orc_u01fixedpt_f32(r["input"])
            assert np.float32(got) == np.float32(exp), r
        else:
            got = L.orc_u01fixedpt_f64(r["input"])
            assert abs(got - exp) <= 2e-16 * max(1.0, abs(exp)), r


def test_u01_exhaustive_direction_and_init(orc):
    # u01fixedpt<float>(r) < 0.5  <=>  r < 2^31 (the proposal direction the
    # kernels read from the top bit); checked on a dense sample of r
    L = orc.lib()
    rs = np.unique(np.concatenate([np.arange(0, 1 << 32, 65537, dtype=np.uint64),
                                   np.array([0x7FFFFFFF, 0x80000000, 0x7FFFFF00, 0x800000FF], np.uint64)]))
    for r in rs[:: max(1, len(rs) // 4000)]:
        r = int(r)
        assert (L.orc_u01fixedpt_f32(r) < 0.5) == (r < (1 << 31))


def test_init_spin_integer_thresholds():
    """The device forms the reference's initial spin (u < 1/3.0) +
    (u < 2/3.0) - 1 (u = u01fixedpt<float>(r) compared in double,
    muca_delta_multigpu.cu:350) as k <= kInitThird and k <= kInitTwoThirds on
    k = 1 | (r >> 8); the same for every one of the 2^24 values of k."""
    import re
    src = open(os.path.join(os.path.dirname(GOLD), "..", "muca_gb300", "csrc", "muca_device.cuh")).read()
    m = re.search(r"kInitThird = (\d+)u, kInitTwoThirds = (\d+)u", src)
    assert m, "thresholds not found in muca_device.cuh"
    t1, t2 = int(m.group(1)), int(m.group(2))
    k = np.arange(1 << 24, dtype=np.uint32) | np.uint32(1)
    u = (k.astype(np.float32) * np.float32(2.0 ** -24)).astype(np.float64)
    assert np.array_equal(u < 1.0 / 3.0, k <= t1)
    assert np.array_equal(u < 2.0 / 3.0, k <= t2)


def test_acceptance_logf_table_lookup(orc):
    """The table path of the acceptance logarithm: entry r >> 9 holds the value
    for u01fixedpt<float>(r) = (2k+1) 2^-24, so a table of libm's values
    reproduces the libm path exactly, and a planted table changes decisions."""
    L = orc.lib()
    rng = np.random.default_rng(5)
    for r in rng.integers(0, 1 << 32, 20000, dtype=np.uint64):
        r = int(r)
        assert np.float32(L.orc_u01fixedpt_f32(r)) == np.float32((2 * (r >> 9) + 1) * 2.0 ** -24)
    tab = np.empty(1 << 23, np.float32)
    L.orc_libm_logf_table(tab)
    Ls, n = 8, 16
    N = Ls * Ls
    w32 = (np.cumsum(rng.normal(-0.9, 0.3, N + 1))).astype(np.float32)
    lat0 = orc.init_lattice(Ls, n, orc.scheme_weight(0, 0))
    ej0, ed0, _ = orc.energies(Ls, lat0)
    outs = []
    for t in (None, tab, np.full(1 << 23, -np.inf, np.float32)):
        L.orc_set_logf_table(None if t is None else t.ctypes.data)
        try:
            ej, ed = ej0.copy(), ed0.copy()
            lat, h = orc.weight_sweep(Ls, lat0.copy(), ej, ed, w32, 3, 100, N, 4 * N)
        finally:
            L.orc_set_logf_table(None)
        outs.append((lat, h, ed))
    for a, b in zip(outs[0], outs[1]):
        np.testing.assert_array_equal(a, b)
    assert not np.array_equal(outs[0][1], outs[2][1])


def test_sweep_tables(orc):
    for L in (2, 4, 6, 8, 72):
        nv, ix = orc.tables(L)
        N = L * L
        assert sorted(ix.tolist()) == list(range(N))
        assert ix[: N // 2].tolist() == list(range(0, N, 2))
        for i in range(N):
            r, c = divmod(i, L)
            assert nv[4 * i] == r * L + (c + 1) % L
            assert nv[4 * i + 1] == r * L + (c - 1) % L
            assert nv[4 * i + 2] == ((r + 1) % L) * L + c
            assert nv[4 * i + 3] == ((r - 1) % L) * L + c


def _prod_cpu(orc, z, ci):
    L, worker, seed, it, therm, nup = map(int, z["pc_cases"][ci])
    N = L * L
    lat = z["pc%d_lat_in" % ci].copy()
    ej, ed, mg = (np.array([v], np.int32) for v in z["pc%d_in" % ci])
    h = np.zeros((N + 1) * (N + 2) // 2, np.uint64)
    orc.lib().orc_produce_cpu_mcs(L, worker, lat, ej, ed, mg, z["pc%d_w" % ci].copy(), h, it, seed, therm, nup)
    return lat, (ej[0], ed[0], mg[0]), h


def test_produce_cpu_mcs_golden(orc):
    z = np.load(os.path.join(GOLD, "ref_cpu.npz"))
    for ci in range(len(z["pc_cases"])):
        lat, st, h = _prod_cpu(orc, z, ci)
        np.testing.assert_array_equal(lat, z["pc%d_lat_out" % ci])
        assert list(st) == list(z["pc%d_out" % ci])
        np.testing.assert_array_equal(h, z["pc%d_hist" % ci])


def test_muca_mag_mcs_golden(orc):
    z = np.load(os.path.join(GOLD, "ref_cpu.npz"))
    for ci in range(len(z["mm_cases"])):
        L, worker, seed, it, therm, nup = map(int, z["mm_cases"][ci])
        N = L * L
        lat = z["mm%d_lat_in" % ci].copy()
        ej, ed = (np.array([v], np.int32) for v in z["mm%d_in" % ci])
        h = np.zeros(N + 1, np.uint64)
        orc.lib().orc_muca_mag_mcs(L, worker, lat, ej, ed, z["mm%d_w" % ci].copy(), h, it, seed, therm, nup)
        np.testing.assert_array_equal(lat, z["mm%d_lat_out" % ci])
        assert [ej[0], ed[0]] == list(z["mm%d_out" % ci])
        np.testing.assert_array_equal(h, z["mm%d_hist" % ci])


def test_hostmath_golden(orc):
    z = np.load(os.path.join(GOLD, "ref_hostmath.npz"))
    Lb = orc.lib()
    for ci in range(4):
        h = z["h%d" % ci]
        assert orc.hist_range(h) == tuple(z["range%d" % ci])
        np.testing.assert_allclose(orc.kull_leibler(h), z["kl%d" % ci][0], rtol=1e-14)
        w, pa = z["w%d" % ci].copy(), z["pacc%d" % ci].copy()
        s, e = orc.hist_range(h)
        Lb.orc_weight_recursion(h, len(h) - 1, pa, s, e, w)
        np.testing.assert_allclose(w, z["rec_w%d" % ci], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(pa, z["rec_pacc%d" % ci], rtol=1e-14)
    for ci in range(3):
        a, e = orc.jackknife(z["jk_x%d" % ci])
        np.testing.assert_allclose([a, e], z["jk%d" % ci], rtol=1e-13)
    for ci in range(2):
        M0, S0, beta, delta, L = z["ob_res%d" % ci]
        N = int(L) ** 2
        l2 = z["ob_lnw%d" % ci].copy()
        Lb.orc_weight_shift(beta, delta, N, l2)
        np.testing.assert_array_equal(l2, z["ob_shifted%d" % ci])
        o = orc.observables(beta, N, z["ob_h%d" % ci], z["ob_boltz%d" % ci])
        np.testing.assert_allclose(o[:2], [M0, S0], rtol=1e-12)


def test_jackknife_single_block_is_nan(orc):
    # the reference divides by JACKS-1; one block gives NaN error (produce2_multigpu.cu:525)
    a, e = orc.jackknife(np.array([0.7]))
    assert a == 0.7 and np.isnan(e)


def _produce_main_restated(orc, L, rng_, jacks, therm_mult, nup_mult, delta0, gap, lnw):
    """produce.cpp main() (:44-269) for one rank, restated from oracle routines."""
    Lb = orc.lib()
    N = L * L
    beta = 2.0
    hist = np.zeros((N + 1) * (N + 2) // 2, np.uint64)  # calloc'ed once, partially zeroed by mcs
    lnw = lnw.copy()
    delta = delta0
    lines = []
    for l in range(rng_):
        lat = orc.init_lattice(L, 1, Lb.orc_scheme_produce_cpu(l)).reshape(-1).copy()
        ej, ed, mg = (np.array([v], np.int32) for v in (x[0] for x in orc.energies(L, lat[None, :])))
        delta = delta + gap / rng_
        Lb.orc_weight_shift(beta, delta, N, lnw)
        bz = np.zeros(N + 1)
        Lb.orc_boltz(beta, delta, N, lnw, bz, 1)
        Lb.orc_produce_cpu_mcs(L, 0, lat, ej, ed, mg, lnw, hist, l, 100 + 1000, N * therm_mult, 0)
        mj, sj = [], []
        for k in range(jacks):
            Lb.orc_produce_cpu_mcs(L, 0, lat, ej, ed, mg, lnw, hist, l, k, 0, N * nup_mult)
            o = orc.observables(beta, N, hist, bz)
            mj.append(o[0])
            sj.append(o[1])
        lines.append((orc.jackknife(mj), orc.jackknife(sj)))
    return lines


def test_produce_main_golden(orc):
    g = json.load(open(os.path.join(GOLD, "ref_produce_main.json")))
    L, rng_, jacks, tm, nm = (int(x) for x in g["args"][:5])
    delta0, gap = float(g["args"][5]), float(g["args"][6])
    lnw = np.array([float(line.split()[1]) for line in g["weight_file"].strip().splitlines()])
    got = _produce_main_restated(orc, L, rng_, jacks, tm, nm, delta0, gap, lnw)
    rows = [list(map(float, ln.split())) for ln in g["observables_file"].strip().splitlines()[1:]]
    assert len(rows) == rng_
    for (m, s), row in zip(got, rows):
        np.testing.assert_allclose([m[0], m[1], s[0], s[1]], row[1:], rtol=2e-9, atol=1e-12)


# ---- live comparisons where the reference harness is built (this checkout) ----

def test_oracle_vs_reference_harness_random(orc):
    R = orc.reflib()
    G = orc.gpuhost()
    if R is None or G is None:
        pytest.skip("reference harness not built here (oracle/_ref)")
    rng = np.random.default_rng(11)
    Lb = orc.lib()
    for L in (4, 6, 10):
        N = L * L
        nv, ix = orc.tables(L)
        for trial in range(3):
            lat = rng.integers(-1, 2, N).astype(np.int8)
            w = rng.normal(0, 1.5, N + 1)
            ej, ed, mg = (np.array([v[0]], np.int32) for v in orc.energies(L, lat[None, :]))
            a = lat.copy()
            h1 = np.zeros((N + 1) * (N + 2) // 2, np.uint64)
            Lb.orc_produce_cpu_mcs(L, trial, a, ej, ed, mg, w, h1, trial, 3, 17, 333)
            b = lat.astype(np.int32)
            h2 = np.zeros_like(h1)
            e2, d2, m2 = C.c_int(int(orc.energies(L, lat[None, :])[0][0])), C.c_int(int((lat * lat).sum())), \
                C.c_int(int(lat.sum()))
            R.refp_mcs(L, trial, b, h2, w.copy(), C.byref(d2), C.byref(e2), C.byref(m2), trial, 3, 17, 333,
                       ix.astype(np.int32), nv.astype(np.int32))
            np.testing.assert_array_equal(a, b.astype(np.int8))
            np.testing.assert_array_equal(h1, h2)
            assert (ej[0], ed[0], mg[0]) == (e2.value, d2.value, m2.value)
