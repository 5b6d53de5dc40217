"""The drop-in executables multigpu_weight and produce_gpu: command line,
output files and their contents against the oracle's restatement of the
reference programs' main loops (muca_delta_multigpu.cu:87-546,
produce2_multigpu.cu:91-363)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "muca_gb300", "_build")


@pytest.fixture(scope="module")
def exes():
    from muca_gb300 import build as b
    b.build()
    return os.path.join(BIN, "multigpu_weight"), os.path.join(BIN, "produce_gpu")


def test_usage_and_bad_arguments(exes):
    for exe in exes:
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([exes[0], "8", "1", "0", "1", "1", "0", "0"], capture_output=True, text=True)
    assert r.returncode == 2  # last_gpu < starting_gpu


def test_no_gpu_fails_loudly(exes, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([exes[0], "8", "0", "0", "1", "1", "0", "0", "--max-iter=2"], capture_output=True,
                       text=True, cwd=tmp_path)
    assert r.returncode == 1 and "error" in r.stderr


@pytest.mark.gpu
def test_multigpu_weight_matches_oracle(exes, orc, tmp_path):
    L, NW, jacks = 4, 256, 2
    N = L * L
    r = subprocess.run([exes[0], str(L), "0", "0", str(jacks), "1", "0", "0", "--chains=%d" % NW,
                        "--max-iter=3000"], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stderr
    d = tmp_path / "fss" / ("L%d" % L)
    files = sorted(os.listdir(d))
    # the reference appends each jack's log name to one stringstream (:327,367),
    # so only jack 0's log can be opened; the weight file is written per jack
    short = [f for f in files if f.startswith("shortiter")]
    assert short == ["shortiter_gpu1_T050c%d_M1_therm1N_Jack0_iterupdate1.01_rand.txt" % NW]
    lines = (d / short[0]).read_text().splitlines()
    assert lines[0] == "#iter width D_KL mcs_time memcpy_time accumulated_time NUPDATES acc_NUP"
    rows = [ln.split() for ln in lines[1:]]

    # oracle: jack 0 then jack 1 with the weights and width carried over
    o = orc.WeightOpts(L=L, nchains=NW, jack=0, gpu=0, starting_M=1, recursive=0, hold_until_full=0,
                       flat_minmean=0, max_iter=3000, rounds=7, nthreads=8, width_start=0)
    lnw = np.zeros(N + 1)
    pacc = np.zeros(N + 1)
    rec = np.zeros(5 * 3000)
    conv = ctypes.c_int()
    lat = orc.init_lattice(L, NW, orc.scheme_weight(0, 0)).reshape(-1).copy()
    ej, ed, _ = orc.energies(L, lat.reshape(NW, N))
    it = orc.lib().orc_weight_run(ctypes.byref(o), lat, ej, ed, lnw, pacc, rec, 3000, ctypes.byref(conv))
    assert conv.value == 1
    assert len(rows) == it
    rec = rec.reshape(-1, 5)
    for k, row in enumerate(rows):
        assert int(row[0]) == k
        assert int(row[1]) == int(rec[k, 0])
        np.testing.assert_allclose(float(row[2]), rec[k, 1], rtol=2e-5)
        assert int(row[6]) == int(rec[k, 2]) and int(row[7]) == int(rec[k, 3])
    w0 = np.loadtxt(d / ("weight_gpu1_T050c%d_M1_therm1N_JACK0_DKL1e-4_iterupdate1.01_rand.txt" % NW))
    np.testing.assert_array_equal(w0[:, 0], np.arange(N + 1))
    np.testing.assert_allclose(w0[:, 1], lnw, rtol=1e-9, atol=1e-9)
    # jack 1: fresh chains (key 10W + 2), weights and width of jack 0
    o.jack = 1
    o.width_start = N
    lat = orc.init_lattice(L, NW, orc.scheme_weight(1, 0)).reshape(-1).copy()
    ej, ed, _ = orc.energies(L, lat.reshape(NW, N))
    orc.lib().orc_weight_run(ctypes.byref(o), lat, ej, ed, lnw, pacc, rec, 3000, ctypes.byref(conv))
    w1 = np.loadtxt(d / ("weight_gpu1_T050c%d_M1_therm1N_JACK1_DKL1e-4_iterupdate1.01_rand.txt" % NW))
    np.testing.assert_allclose(w1[:, 1], lnw, rtol=1e-9, atol=1e-9)
    res = [f for f in files if f.startswith("converge_result")]
    assert res == ["converge_result_gpu1_T050c%dM1_therm1N_iterupdate1.01_rand.txt" % NW]
    assert "D_KL is below 1e-4" in r.stdout and "E_DELTA : " in r.stdout


def _produce_restated(orc, L, NW, ndev, rng_, tm, nm, delta0, gap, lnw_file):
    """produce2_multigpu.cu main (:91-363) restated with oracle routines."""
    return [(m, s) for m, s, _ in _produce_variants(orc, L, NW, ndev, rng_, 0, tm, nm, delta0, gap, lnw_file)]


def _produce_variants(orc, L, NW, ndev, rng_, jacks, tm, nm, delta0, gap, lnw_file, blocks=False, reuse=False,
                      start_lats=None):
    """The production loop with the options of produce_gpu: `blocks`
    jackknifes over `jacks` production blocks (seeds of the block loop at
    produce2_multigpu.cu:324-347, iter jj, seed 100 + l + 2000 g), `reuse`
    runs the thermalisation and production of the first Delta point only and
    reweights its histograms at every point.  Returns per Delta point the
    jackknifed (<|M|>, chi, U4) as (avg, err) pairs.  `start_lats`
    ([chain][site], NW * ndev chains): the chains start there (--load-chains)
    instead of from the reference's initial spins."""
    N = L * L
    beta = 2.0
    lats, ejs, eds, mgs = [], [], [], []
    for g in range(ndev):
        if start_lats is not None:
            lat = np.ascontiguousarray(start_lats[g * NW:(g + 1) * NW], np.int8).copy()
        else:
            lat = orc.init_lattice(L, NW, orc.scheme_produce(g)).copy()
        ej, ed, mg = orc.energies(L, lat)
        lats.append(lat); ejs.append(ej); eds.append(ed); mgs.append(mg)
    deltas, d = [], delta0
    for l in range(rng_):
        d = d + gap / rng_
        deltas.append(d)
    boltz = []
    lnw_host = lnw_file.copy()
    for d in deltas:
        orc.lib().orc_weight_shift(beta, d, N, lnw_host)
        bz = np.zeros(N + 1)
        orc.lib().orc_boltz(beta, d, N, lnw_host, bz, 0)
        boltz.append(bz)
    nu = jacks if blocks else ndev
    q = np.zeros((rng_, nu, 3))
    sums = np.zeros((rng_, nu, 4))
    for l in range(1 if reuse else rng_):
        for g in range(ndev):
            lats[g], _ = orc.produce_sweep(L, lats[g], ejs[g], eds[g], mgs[g], lnw_file, 0, 100 + 1000 * g + l,
                                           N * tm, 0, nthreads=8)
        pts = range(rng_) if reuse else [l]
        for u in range(nu):
            for g in (range(ndev) if blocks else [u]):
                it, seed = (u, 100 + l + 2000 * g) if blocks else (l, 100 + 2000 * g)
                lats[g], h = orc.produce_sweep(L, lats[g], ejs[g], eds[g], mgs[g], lnw_file, it, seed, 0, N * nm,
                                               nthreads=8)
                for k in pts:
                    o = orc.observables(beta, N, h, boltz[k])
                    q[k, u] = o[:3]
                    sums[k, u] += o[3:]
    if blocks:
        s, m1, m2, m4 = (sums[..., i] for i in range(4))
        q[..., 0] = m1 / s
        q[..., 1] = (m2 / s - (m1 / s) ** 2) * beta / N
        q[..., 2] = 1.0 - (m4 / s) / (3.0 * (m2 / s) ** 2)
    return [tuple(orc.jackknife(q[k, :, i]) for i in range(3)) for k in range(rng_)]


@pytest.mark.gpu
def test_produce_gpu_matches_oracle(exes, orc, tmp_path):
    L, NW, ndev, rng_, tm, nm = 4, 256, 2, 3, 20, 40
    N = L * L
    d = tmp_path / "fss" / ("L%d" % L)
    d.mkdir(parents=True)
    rng = np.random.default_rng(9)
    lnw = np.cumsum(rng.normal(-0.8, 0.4, N + 1))
    lnw -= lnw[0]
    with open(d / "weight_mpi_T050c16_M200_JACK0_DKL1e-4.txt", "w") as f:
        for i, v in enumerate(lnw):
            f.write("%d %.10g\n" % (i, v))
    lnw_file = np.array([float("%.10g" % v) for v in lnw])
    args = [str(L), "0", str(ndev - 1), str(rng_), "5", str(tm), str(nm), "1.9", "0.1"]
    r = subprocess.run([exes[1]] + args + ["--chains=%d" % NW], capture_output=True, text=True, cwd=tmp_path,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    name = "observables_gpu%d_T050_JACKgpu_THERM%sN_NUP%sN_delta1.9to0.1noreset.txt" % (ndev, tm, nm)
    rows = [list(map(float, ln.split())) for ln in (d / name).read_text().splitlines()]
    exp = _produce_restated(orc, L, NW, ndev, rng_, tm, nm, 1.9, 0.1, lnw_file)
    assert len(rows) == rng_
    for i, ((m, s), row) in enumerate(zip(exp, rows)):
        # the first line's Delta is printed with the stream's default 6 digits,
        # later lines with the 10 digits set by the first line's setprecision
        np.testing.assert_allclose(row[0], 1.9 + 0.1 * (i + 1) / rng_, rtol=1e-5 if i == 0 else 1e-9)
        np.testing.assert_allclose(row[1:], [m[0], m[1], s[0], s[1]], rtol=2e-9, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("opts", [["--jack-blocks", "--binder"], ["--reuse-histogram", "--binder"],
                                  ["--reuse-histogram", "--jack-blocks"]])
def test_produce_gpu_options_match_oracle(exes, orc, tmp_path, opts):
    L, NW, ndev, rng_, jacks, tm, nm = 4, 128, 2, 3, 3, 10, 30
    N = L * L
    d = tmp_path / "fss" / ("L%d" % L)
    d.mkdir(parents=True)
    rng = np.random.default_rng(11)
    lnw = np.cumsum(rng.normal(-0.8, 0.4, N + 1))
    lnw -= lnw[0]
    with open(d / "weight_mpi_T050c16_M200_JACK0_DKL1e-4.txt", "w") as f:
        for i, v in enumerate(lnw):
            f.write("%d %.10g\n" % (i, v))
    lnw_file = np.array([float("%.10g" % v) for v in lnw])
    args = [str(L), "0", str(ndev - 1), str(rng_), str(jacks), str(tm), str(nm), "1.9", "0.1"]
    r = subprocess.run([exes[1]] + args + ["--chains=%d" % NW] + opts, capture_output=True, text=True,
                       cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stderr
    exp = _produce_variants(orc, L, NW, ndev, rng_, jacks, tm, nm, 1.9, 0.1, lnw_file,
                            blocks="--jack-blocks" in opts, reuse="--reuse-histogram" in opts)
    name = "observables_gpu%d_T050_JACKgpu_THERM%sN_NUP%sN_delta1.9to0.1noreset.txt" % (ndev, tm, nm)
    rows = [list(map(float, ln.split())) for ln in (d / name).read_text().splitlines()]
    assert len(rows) == rng_
    for (m, s, _), row in zip(exp, rows):
        assert np.all(np.isfinite(row))
        np.testing.assert_allclose(row[1:], [m[0], m[1], s[0], s[1]], rtol=2e-9, atol=1e-12)
    if "--binder" in opts:
        bname = "observables_binder_gpu%d_T050_THERM%sN_NUP%sN_delta1.9to0.1.txt" % (ndev, tm, nm)
        lines = (d / bname).read_text().splitlines()
        assert lines[0].startswith("#")
        brows = [list(map(float, ln.split())) for ln in lines[1:]]
        assert len(brows) == rng_
        for (_, _, u), row in zip(exp, brows):
            np.testing.assert_allclose(row[1:], [u[0], u[1]], rtol=2e-9, atol=1e-12)


@pytest.mark.gpu
def test_produce_gpu_reuse_first_point_is_the_plain_run(exes, tmp_path):
    L, NW, ndev, rng_, tm, nm = 8, 256, 1, 4, 10, 20
    N = L * L
    outs = []
    for k, extra in enumerate([[], ["--reuse-histogram"]]):
        d = tmp_path / str(k) / "fss" / ("L%d" % L)
        d.mkdir(parents=True)
        with open(d / "weight_mpi_T050c16_M200_JACK0_DKL1e-4.txt", "w") as f:
            for i in range(N + 1):
                f.write("%d %.10g\n" % (i, -0.9 * i))
        args = [str(L), "0", str(ndev - 1), str(rng_), "2", str(tm), str(nm), "1.5", "0.4"]
        r = subprocess.run([exes[1]] + args + ["--chains=%d" % NW] + extra, capture_output=True, text=True,
                           cwd=tmp_path / str(k), timeout=600)
        assert r.returncode == 0, r.stderr
        name = "observables_gpu%d_T050_JACKgpu_THERM%sN_NUP%sN_delta1.5to0.4noreset.txt" % (ndev, tm, nm)
        outs.append((d / name).read_text().splitlines())
    assert outs[0][0] == outs[1][0]
    assert outs[0][1:] != outs[1][1:]


def _weight_oracle(orc, L, NW, lnw0, recursive, max_iter):
    o = orc.WeightOpts(L=L, nchains=NW, jack=0, gpu=0, starting_M=1, recursive=recursive, hold_until_full=0,
                       flat_minmean=0, max_iter=max_iter, rounds=7, nthreads=8, width_start=0)
    N = L * L
    lnw = np.array(lnw0, np.float64)
    pacc = np.zeros(N + 1)
    rec = np.zeros(5 * max_iter)
    conv = ctypes.c_int()
    lat = orc.init_lattice(L, NW, orc.scheme_weight(0, 0)).reshape(-1).copy()
    ej, ed, _ = orc.energies(L, lat.reshape(NW, N))
    it = orc.lib().orc_weight_run(ctypes.byref(o), lat, ej, ed, lnw, pacc, rec, max_iter, ctypes.byref(conv))
    return it, bool(conv.value), rec.reshape(-1, 5)[:it], lnw


def _check_log(rows, it, rec):
    assert len(rows) == it
    for k, row in enumerate(rows):
        assert int(row[0]) == k
        assert int(row[1]) == int(rec[k, 0])
        np.testing.assert_allclose(float(row[2]), rec[k, 1], rtol=2e-5)
        assert int(row[6]) == int(rec[k, 2]) and int(row[7]) == int(rec[k, 3])


@pytest.mark.gpu
def test_multigpu_weight_continuing_matches_oracle(exes, orc, tmp_path):
    """continuing=1: the weights start from initweight_L128_T050.txt (one value
    per line, muca_delta_multigpu.cu:223-235), the files carry the
    extrapolated-init names."""
    L, NW = 4, 256
    N = L * L
    d = tmp_path / "fss" / ("L%d" % L)
    d.mkdir(parents=True)
    w0 = -1.7 * np.arange(N + 1) + 0.05 * np.arange(N + 1) ** 2
    (d / "initweight_L128_T050.txt").write_text("".join("%.17g\n" % v for v in w0))
    r = subprocess.run([exes[0], str(L), "0", "0", "1", "1", "0", "1", "--chains=%d" % NW, "--max-iter=3000"],
                       capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stderr
    it, conv, rec, lnw = _weight_oracle(orc, L, NW, w0, 0, 3000)
    rows = [ln.split() for ln in (d / ("shortiter_gpu1_T050c%d_M1_therm1N_Jack0_extrapolated1.txt" % NW))
            .read_text().splitlines()[1:]]
    _check_log(rows, it, rec)
    assert conv
    w = np.loadtxt(d / ("weight_gpu1_T050c%d_M1_therm1N_JACK0_DKL1e-4_fromextrapolatedinit1.txt" % NW))
    np.testing.assert_allclose(w[:, 1], lnw, rtol=1e-9, atol=1e-9)


@pytest.mark.gpu
def test_multigpu_weight_recursion_matches_oracle(exes, orc, tmp_path):
    """recursive_update=1: weight_recursion after every iteration (the
    reference parses the flag but never calls it); the iteration log follows
    the oracle's recursion step for step."""
    L, NW, K = 4, 256, 60
    r = subprocess.run([exes[0], str(L), "0", "0", "1", "1", "1", "0", "--chains=%d" % NW, "--max-iter=%d" % K],
                       capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stderr
    N = L * L
    it, conv, rec, _ = _weight_oracle(orc, L, NW, np.zeros(N + 1), 1, K)
    d = tmp_path / "fss" / ("L%d" % L)
    rows = [ln.split() for ln in (d / ("shortiter_gpu1_T050c%d_M1_therm1N_Jack0_iterupdate1.01_rand.txt" % NW))
            .read_text().splitlines()[1:]]
    _check_log(rows, it, rec)


# ---- malformed weight files (host side, before any device work) ------------------------------

def _weight_pairs(L, lnw):
    return "".join("%d %.10g\n" % (i, v) for i, v in enumerate(lnw))


@pytest.mark.parametrize("case", ["missing", "truncated", "non_numeric", "nan", "index", "extra", "empty"])
def test_produce_gpu_rejects_malformed_weight_file(exes, tmp_path, case):
    """The reference reads the weight file unchecked (produce2_multigpu.cu:210-220):
    a missing file prints "!error!" and runs on zero weights, a short or
    non-numeric one leaves zeros, a trailing newline writes past the array.
    The drop-in refuses such a file with status 3 and names the problem,
    before it touches the GPU (so this runs without one)."""
    L = 4
    N = L * L
    d = tmp_path / "fss" / ("L%d" % L)
    d.mkdir(parents=True)
    lnw = -0.5 * np.arange(N + 1)
    body = _weight_pairs(L, lnw)
    lines = body.splitlines(keepends=True)
    if case == "truncated":
        body = "".join(lines[:-3])
    elif case == "non_numeric":
        lines[5] = "5 abc\n"
        body = "".join(lines)
    elif case == "nan":
        lines[7] = "7 nan\n"
        body = "".join(lines)
    elif case == "index":
        lines[3] = "4 -1.5\n"
        body = "".join(lines)
    elif case == "extra":
        body = body + "%d 0\n" % (N + 1)
    elif case == "empty":
        body = "\n"
    if case != "missing":
        (d / "weight_mpi_T050c16_M200_JACK0_DKL1e-4.txt").write_text(body)
    args = [str(L), "0", "0", "1", "1", "1", "1", "1.9", "0.1", "--chains=64"]
    r = subprocess.run([exes[1]] + args, capture_output=True, text=True, cwd=tmp_path, timeout=120)
    assert r.returncode == 3, (r.returncode, r.stderr)
    assert "weight file" in r.stderr
    expect = {"missing": "cannot open", "truncated": "entries, expected N+1 = 17", "non_numeric": "'abc'",
              "nan": "'nan'", "index": "index '4' (expected 3)", "extra": "more than N+1",
              "empty": "0 entries"}[case]
    assert expect in r.stderr, r.stderr


@pytest.mark.parametrize("case", ["truncated", "non_numeric", "missing"])
def test_multigpu_weight_rejects_malformed_initial_weight(exes, tmp_path, case):
    """The continuing path's initial weight (one value per line,
    muca_delta_multigpu.cu:223-235) must hold N+1 finite values."""
    L = 4
    N = L * L
    d = tmp_path / "fss" / ("L%d" % L)
    d.mkdir(parents=True)
    vals = ["%.10g" % (-0.25 * i) for i in range(N + 1)]
    if case == "truncated":
        vals = vals[:N]
    elif case == "non_numeric":
        vals[2] = "x1"
    if case != "missing":
        (d / "initweight_L128_T050.txt").write_text("\n".join(vals) + "\n")
    r = subprocess.run([exes[0], str(L), "0", "0", "1", "1", "0", "1", "--chains=64", "--max-iter=2"],
                       capture_output=True, text=True, cwd=tmp_path, timeout=120)
    assert r.returncode == 3, (r.returncode, r.stderr)
    expect = {"truncated": "16 values, expected N+1 = 17", "non_numeric": "'x1'", "missing": "cannot open"}[case]
    assert expect in r.stderr, r.stderr


# ---- chain files: production from a weight run's final lattices --------------------------------

def _chain_file(path, L, n, lat=None, magic=b"MUCACHN1", extra=b""):
    import struct
    if lat is None:
        lat = np.zeros((n, L * L), np.int8)
    with open(path, "wb") as f:
        f.write(magic + struct.pack("<II", L, n) + np.ascontiguousarray(lat, np.int8).tobytes() + extra)


def _read_chain_file(path):
    import struct
    b = open(path, "rb").read()
    assert b[:8] == b"MUCACHN1"
    L, n = struct.unpack("<II", b[8:16])
    lat = np.frombuffer(b[16:], np.int8).reshape(n, L * L)
    return L, n, lat


@pytest.mark.parametrize("case", ["missing", "magic", "size", "truncated", "spin"])
def test_produce_gpu_rejects_bad_chain_file(exes, tmp_path, case):
    """--load-chains is checked before any device work (no GPU needed): the
    file must hold exactly chains x N spins in {-1, 0, 1} for this L and
    chain count, after the header."""
    L, NW = 4, 64
    N = L * L
    d = tmp_path / "fss" / ("L%d" % L)
    d.mkdir(parents=True)
    (d / "weight_mpi_T050c16_M200_JACK0_DKL1e-4.txt").write_text(_weight_pairs(L, -0.5 * np.arange(N + 1)))
    cf = tmp_path / "chains.bin"
    if case == "magic":
        _chain_file(cf, L, NW, magic=b"NOTCHAIN")
    elif case == "size":
        _chain_file(cf, L, NW + 1)
    elif case == "truncated":
        _chain_file(cf, L, NW)
        cf.write_bytes(cf.read_bytes()[:-5])
    elif case == "spin":
        lat = np.zeros((NW, N), np.int8)
        lat[3, 7] = 2
        _chain_file(cf, L, NW, lat)
    args = [str(L), "0", "0", "1", "1", "1", "1", "1.9", "0.1", "--chains=%d" % NW, "--load-chains=%s" % cf]
    r = subprocess.run([exes[1]] + args, capture_output=True, text=True, cwd=tmp_path, timeout=120)
    assert r.returncode == 3, (r.returncode, r.stderr)
    expect = {"missing": "cannot open", "magic": "not a chain file", "size": "expected 64 of L=4",
              "truncated": "truncated", "spin": "not in {-1, 0, 1}"}[case]
    assert "chain file" in r.stderr and expect in r.stderr, r.stderr


@pytest.mark.gpu
def test_weight_run_chains_start_production(exes, orc, tmp_path):
    """multigpu_weight --save-chains writes the chains' final lattices;
    produce_gpu --load-chains starts from them.  The observables equal the
    reference production loop restated with the oracle from those lattices."""
    L, NW, jacks, rng_, tm, nm = 8, 128, 4, 2, 5, 20
    N = L * L
    cf = tmp_path / "chains.bin"
    r = subprocess.run([exes[0], str(L), "0", "0", "1", "64", "0", "0", "--chains=%d" % NW, "--flat=minmean",
                        "--max-iter=3000", "--save-chains=%s" % cf], capture_output=True, text=True, cwd=tmp_path,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    Lc, n, lat = _read_chain_file(cf)
    assert (Lc, n) == (L, NW) and set(np.unique(lat)) <= {-1, 0, 1}
    d = tmp_path / "fss" / ("L%d" % L)
    wfile = [f for f in os.listdir(d) if f.startswith("weight_gpu1_")][0]
    txt = (d / wfile).read_text()
    (d / "weight_mpi_T050c16_M200_JACK0_DKL1e-4.txt").write_text(txt)
    lnw_file = np.array([float(line.split()[1]) for line in txt.strip().splitlines()])
    args = [str(L), "0", "0", str(rng_), str(jacks), str(tm), str(nm), "1.9", "0.1", "--chains=%d" % NW,
            "--jack-blocks", "--load-chains=%s" % cf]
    r = subprocess.run([exes[1]] + args, capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stderr
    name = "observables_gpu1_T050_JACKgpu_THERM%sN_NUP%sN_delta1.9to0.1noreset.txt" % (tm, nm)
    rows = [list(map(float, ln.split())) for ln in (d / name).read_text().splitlines()]
    exp = _produce_variants(orc, L, NW, 1, rng_, jacks, tm, nm, 1.9, 0.1, lnw_file, blocks=True,
                            start_lats=lat)
    assert len(rows) == rng_
    for (m, s_, _), row in zip(exp, rows):
        assert np.all(np.isfinite(row[1:]))
        np.testing.assert_allclose(row[1:], [m[0], m[1], s_[0], s_[1]], rtol=2e-9, atol=1e-12)


@pytest.mark.gpu
def test_multigpu_weight_hist_dump(exes, tmp_path):
    """--hist-dump writes each jack's final weights beside its last
    iteration's histogram, in the reference's commented-out format
    (muca_delta_multigpu.cu:528-541): the weights equal the weight file's,
    and every chain contributed the same number of entries."""
    L, NW = 4, 256
    N = L * L
    r = subprocess.run([exes[0], str(L), "0", "0", "1", "1", "0", "0", "--chains=%d" % NW, "--max-iter=3000",
                        "--hist-dump"], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stderr
    d = tmp_path / "fss" / ("L%d" % L)
    rows = [ln.split(" ") for ln in (d / "E_Delta_multi_T050_JACK0.txt").read_text().splitlines()]
    assert [int(x[0]) for x in rows] == list(range(N + 1))
    h = np.array([int(x[2]) for x in rows], np.uint64)
    assert int(h.sum()) > 0 and int(h.sum()) % NW == 0
    wfiles = [f for f in os.listdir(d) if f.startswith("weight_gpu1_")]
    if wfiles:  # written on convergence, from the same final weights
        wrows = [ln.split(" ") for ln in (d / wfiles[0]).read_text().splitlines()]
        assert [x[1] for x in rows] == [x[1] for x in wrows]
