"""Generate the golden fixtures under tests/golden/ from the reference.

Run in a checkout where the reference is available ($MUCA_REFERENCE, else
the REF of oracle/Makefile) after `make -C oracle ref`:

    python tests/golden/make_golden.py

Fixtures written (all small):
  philox_kat.json      Random123/examples/kat_vectors:24-29 (philox4x32, 7 and 10 rounds)
  u01_kat.json         Random123/examples/ut_uniform_kat_vectors.dat, the
                       u01fixedpt<float|double>(uint32) entries
  ref_cpu.npz          outputs of the reference CPU routines compiled from
                       produce.cpp / muca_mag.cpp (oracle/_ref/libref_cpu.so)
  ref_hostmath.npz     outputs of the host routines of muca_delta_multigpu.cu /
                       produce2_multigpu.cu (oracle/_ref/libref_gpuhost.so)
  ref_produce_main.json  the observables file written by the reference
                       produce_mpi program (oracle/_ref/produce_mpi, one rank)
                       for a small synthetic weight file
"""
from __future__ import annotations

import ctypes as C
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import orc  # noqa: E402

REF = orc.reference_dir()
if not REF or not os.path.isdir(REF):
    sys.exit("make_golden.py: the reference checkout %r does not exist; set MUCA_REFERENCE" % REF)


def philox_kat():
    rows = []
    with open(os.path.join(REF, "Random123/examples/kat_vectors")) as f:
        for ln, line in enumerate(f, 1):
            t = line.split()
            if len(t) == 12 and t[0] == "philox4x32":
                rows.append({"line": ln, "rounds": int(t[1]), "ctr": [int(x, 16) for x in t[2:6]],
                             "key": [int(x, 16) for x in t[6:8]], "out": [int(x, 16) for x in t[8:12]]})
    return rows


def u01_kat():
    pat = re.compile(r'insert\("(u01fixedpt<(float|double)>)\((minu32|mini32|maxu32|maxi32) \+ (u?int32_t)\(a\)\) '
                     r'a=(-?\d+)", ([-0-9.e+]+)L\);')
    base = {"minu32": 0, "maxu32": 0xFFFFFFFF, "mini32": -(1 << 31), "maxi32": (1 << 31) - 1}
    rows = []
    with open(os.path.join(REF, "Random123/examples/ut_uniform_kat_vectors.dat")) as f:
        for ln, line in enumerate(f, 1):
            m = pat.search(line)
            if not m:
                continue
            fn, ty, b, _, a, val = m.groups()
            r = (base[b] + int(a)) & 0xFFFFFFFF
            rows.append({"line": ln, "type": ty, "input": r, "value": val})
    return rows


def ref_cpu():
    R = orc.reflib()
    rng = np.random.default_rng(20261203)
    out = {}
    cases = []
    # produce.cpp:421-511 (mcs) on L=4,6,8 with random lattice and weights
    for ci, (L, worker, seed, it, therm, nup) in enumerate([(4, 0, 7, 0, 32, 500), (6, 3, 1000, 5, 36, 777),
                                                            (8, 11, 1100, 2, 64, 2000)]):
        N = L * L
        nv, ix = orc.tables(L)
        lat = rng.integers(-1, 2, N).astype(np.int32)
        w = rng.normal(0, 2, N + 1)
        ej = C.c_int(R.refp_total_energy(L, lat.copy()))
        ed = C.c_int(int((lat * lat).sum()))
        mg = C.c_int(int(lat.sum()))
        out["pc%d_lat_in" % ci] = lat.astype(np.int8)
        out["pc%d_w" % ci] = w
        out["pc%d_in" % ci] = np.array([ej.value, ed.value, mg.value], np.int64)
        h = np.zeros((N + 1) * (N + 2) // 2, np.uint64)
        lat2 = lat.copy()
        R.refp_mcs(L, worker, lat2, h, w.copy(), C.byref(ed), C.byref(ej), C.byref(mg), it, seed, therm, nup,
                   ix.astype(np.int32), nv.astype(np.int32))
        out["pc%d_lat_out" % ci] = lat2.astype(np.int8)
        out["pc%d_out" % ci] = np.array([ej.value, ed.value, mg.value], np.int64)
        out["pc%d_hist" % ci] = h
        cases.append([L, worker, seed, it, therm, nup])
    out["pc_cases"] = np.array(cases, np.int64)
    cases = []
    # muca_mag.cpp:312-393 (mcs, random site, 3 streams)
    for ci, (L, worker, seed, it, therm, nup) in enumerate([(4, 0, 0, 0, 16, 400), (6, 2, 1, 3, 0, 999),
                                                            (8, 5, 0, 7, 100, 3000)]):
        N = L * L
        nv, ix = orc.tables(L)
        lat = rng.integers(-1, 2, N).astype(np.int32)
        w = rng.normal(0, 2, N + 1)
        ej = C.c_int(R.refp_total_energy(L, lat.copy()))
        ed = C.c_int(int((lat * lat).sum()))
        out["mm%d_lat_in" % ci] = lat.astype(np.int8)
        out["mm%d_w" % ci] = w
        out["mm%d_in" % ci] = np.array([ej.value, ed.value], np.int64)
        h = np.zeros(N + 1, np.uint64)
        lat2 = lat.copy()
        R.refm_mcs(L, worker, lat2, h, w.copy(), ix.astype(np.int32), nv.astype(np.int32), C.byref(ej), C.byref(ed),
                   it, seed, therm, nup)
        out["mm%d_lat_out" % ci] = lat2.astype(np.int8)
        out["mm%d_out" % ci] = np.array([ej.value, ed.value], np.int64)
        out["mm%d_hist" % ci] = h
        cases.append([L, worker, seed, it, therm, nup])
    out["mm_cases"] = np.array(cases, np.int64)
    return out


def ref_hostmath():
    G = orc.gpuhost()
    rng = np.random.default_rng(7)
    out = {}
    for ci, N in enumerate([16, 64, 256, 1024]):
        h = rng.integers(0, 60, N + 1).astype(np.uint64)
        h[: ci + 1] = 0
        h[-(ci + 2):] = rng.integers(0, 2, ci + 2).astype(np.uint64)
        if ci == 2:
            h[N // 2: N // 2 + 3] = 0  # a gap inside the range
        s, e = C.c_int(), C.c_int()
        G.refg_hist_range(h, N, C.byref(s), C.byref(e))
        kl = G.refg_kull_leibler(h, N)
        w = rng.normal(0, 3, N + 1)
        pa = rng.uniform(0, 50, N + 1)
        w2, pa2 = w.copy(), pa.copy()
        G.refg_weight_recursion(N, h, pa2, s.value, e.value, w2)
        out["h%d" % ci] = h
        out["range%d" % ci] = np.array([s.value, e.value], np.int64)
        out["kl%d" % ci] = np.array([kl])
        out["w%d" % ci] = w
        out["pacc%d" % ci] = pa
        out["rec_w%d" % ci] = w2
        out["rec_pacc%d" % ci] = pa2
    for ci, J in enumerate([2, 5, 10]):
        x = rng.normal(1, 0.1, J)
        a_, e_ = C.c_double(), C.c_double()
        G.refg_jakknife.argtypes = [np.ctypeslib.ndpointer(np.float64), C.POINTER(C.c_double),
                                    C.POINTER(C.c_double), C.c_uint]
        G.refg_jakknife(x.copy(), C.byref(a_), C.byref(e_), J)
        out["jk_x%d" % ci] = x
        out["jk%d" % ci] = np.array([a_.value, e_.value])
    # weight_shift + observables (produce2_multigpu.cu) on L=4 and L=8 triangles
    for ci, (L, beta, delta) in enumerate([(4, 2.0, 1.96), (8, 2.0, 1.5)]):
        N = L * L
        hs = (N + 1) * (N + 2) // 2
        h2 = rng.integers(0, 1000, hs).astype(np.uint64)
        h2[rng.random(hs) < 0.3] = 0
        lnw = rng.normal(0, 5, N + 1)
        l2 = lnw.copy()
        G.refg_weight_shift(beta, delta, N, l2)
        bz = np.exp(-beta * delta * np.arange(N + 1) - l2)  # produce2_multigpu.cu:297
        Mj, Sj = np.zeros(1), np.zeros(1)
        G.refg_observables(beta, delta, N, h2, bz, l2, Mj, Sj, 0)
        out["ob_h%d" % ci] = h2
        out["ob_lnw%d" % ci] = lnw
        out["ob_shifted%d" % ci] = l2
        out["ob_boltz%d" % ci] = bz
        out["ob_res%d" % ci] = np.array([Mj[0], Sj[0], beta, delta, L])
    return out


def ref_produce_main():
    """Run the reference produce_mpi (one rank) on a synthetic weight file."""
    exe = os.path.join(orc.REFOUT, "produce_mpi")
    L = 4
    N = L * L
    rng = np.random.default_rng(3)
    lnw = np.cumsum(rng.normal(-1.0, 0.3, N + 1))
    lnw -= lnw[0]
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "fss", "L4"))
        with open(os.path.join(d, "fss", "L4", "weight_mpi_T050c16_M200_JACK0_DKL1e-4.txt"), "w") as f:
            for i, v in enumerate(lnw):
                f.write("%d %.10g\n" % (i, v))
        args = ["4", "2", "3", "10", "50", "1.9", "0.1"]  # L range jacks therm_mult nup_mult delta gap
        r = subprocess.run([exe] + args, cwd=d, capture_output=True, text=True, timeout=120)
        files = os.listdir(os.path.join(d, "fss", "L4"))
        obs = [f for f in files if f.startswith("observables")]
        text = open(os.path.join(d, "fss", "L4", obs[0])).read()
        wtext = open(os.path.join(d, "fss", "L4", "weight_mpi_T050c16_M200_JACK0_DKL1e-4.txt")).read()
    return {"args": args, "weight_file": wtext, "observables_file_name": obs[0], "observables_file": text,
            "stdout_rc": r.returncode}


def main():
    orc.build(ref=True)
    with open(os.path.join(HERE, "philox_kat.json"), "w") as f:
        json.dump({"source": "Random123/examples/kat_vectors", "rows": philox_kat()}, f, indent=1)
    with open(os.path.join(HERE, "u01_kat.json"), "w") as f:
        json.dump({"source": "Random123/examples/ut_uniform_kat_vectors.dat", "rows": u01_kat()}, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "ref_cpu.npz"), **ref_cpu())
    np.savez_compressed(os.path.join(HERE, "ref_hostmath.npz"), **ref_hostmath())
    with open(os.path.join(HERE, "ref_produce_main.json"), "w") as f:
        json.dump(ref_produce_main(), f, indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
