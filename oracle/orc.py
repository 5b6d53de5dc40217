"""ctypes binding of the CPU oracle and the reference harness.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py.  The product (muca_gb300) never imports it.

* ``lib()``      -> oracle/_build/liborc.so (CPU restatement, muca_oracle.c)
* ``reflib()``   -> oracle/_ref/libref_cpu.so (produce.cpp / muca_mag.cpp
                    compiled from the reference sources), or None
* ``gpuhost()``  -> oracle/_ref/libref_gpuhost.so (host routines of the
                    reference GPU programs), or None
* ``refgpu()``   -> oracle/_build/librefgpu.so (driver-API launcher of the
                    reference kernels compiled to oracle/_ref/*.cubin), or None
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REFOUT = os.path.join(HERE, "_ref")
REF_WEIGHT_CUBIN = os.path.join(REFOUT, "ref_weight.cubin")
REF_PRODUCE_CUBIN = os.path.join(REFOUT, "ref_produce.cubin")

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_i8p = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


class InitScheme(C.Structure):
    _fields_ = [("key0_mul", C.c_uint32), ("key0_add", C.c_uint32), ("key1", C.c_uint32),
                ("ctr0", C.c_uint32 * 4), ("ctr_word", C.c_uint32), ("rounds", C.c_uint32)]


class WeightOpts(C.Structure):
    _fields_ = [("L", C.c_uint), ("nchains", C.c_uint), ("jack", C.c_uint), ("gpu", C.c_uint),
                ("starting_M", C.c_uint), ("recursive", C.c_int), ("hold_until_full", C.c_int),
                ("flat_minmean", C.c_int), ("max_iter", C.c_uint), ("rounds", C.c_uint),
                ("nthreads", C.c_int), ("width_start", C.c_uint), ("sched", C.c_uint), ("nup_max", C.c_uint),
                ("algo", C.c_uint)]


def reference_dir() -> str:
    """The reference checkout the recipe reads: $MUCA_REFERENCE, else the
    recipe's own REF (oracle/Makefile).  It exists only where the reference
    was checked out; nothing on the GPU host needs it."""
    env = os.environ.get("MUCA_REFERENCE")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], stdout=subprocess.PIPE, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


def build(ref: bool = False, refgpu: bool = False) -> None:
    targets = ["oracle"] + (["refgpu"] if refgpu else []) + (["ref"] if ref else [])
    extra = ["REF=" + os.environ["MUCA_REFERENCE"]] if ref and os.environ.get("MUCA_REFERENCE") else []
    subprocess.run(["make", "-s", "-C", HERE, "-j8"] + targets + extra, check=True)


_LIB = None


def lib():
    global _LIB
    if _LIB is not None:
        return _LIB
    path = os.path.join(BUILD, "liborc.so")
    if not os.path.exists(path):
        build()
    L = C.CDLL(path)
    L.orc_philox4x32.argtypes = [C.c_uint, _u32p, _u32p, _u32p]
    L.orc_u01fixedpt_f32.argtypes = [C.c_uint32]
    L.orc_u01fixedpt_f32.restype = C.c_float
    L.orc_u01fixedpt_f64.argtypes = [C.c_uint32]
    L.orc_u01fixedpt_f64.restype = C.c_double
    L.orc_init_spin.argtypes = [C.c_uint32]
    L.orc_sweep_tables.argtypes = [C.c_uint, _u32p, _u32p]
    for n in ("orc_scheme_weight",):
        getattr(L, n).argtypes = [C.c_uint, C.c_uint]
        getattr(L, n).restype = InitScheme
    for n in ("orc_scheme_produce", "orc_scheme_produce_cpu", "orc_scheme_muca_mag"):
        getattr(L, n).argtypes = [C.c_uint]
        getattr(L, n).restype = InitScheme
    L.orc_init_lattice.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.POINTER(InitScheme), _i8p]
    L.orc_init_lattice_graded.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.POINTER(InitScheme), _i8p]
    L.orc_chain_energies.argtypes = [C.c_uint, C.c_uint, _i8p, _i32p, _i32p, _i32p]
    L.orc_weight_sweep.argtypes = [C.c_uint, C.c_uint, C.c_uint, _i8p, _i32p, _i32p, _f32p, _u64p,
                                   C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint, C.c_int]
    L.orc_produce_sweep.argtypes = [C.c_uint, C.c_uint, C.c_uint, _i8p, _i32p, _i32p, _i32p, _f64p, _u64p,
                                    C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint, C.c_int]
    L.orc_produce_cpu_mcs.argtypes = [C.c_uint, C.c_uint, _i8p, _i32p, _i32p, _i32p, _f64p, _u64p,
                                      C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint64]
    L.orc_muca_mag_mcs.argtypes = [C.c_uint, C.c_uint, _i8p, _i32p, _i32p, _f64p, _u64p,
                                   C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint64]
    L.orc_hist_range.argtypes = [_u64p, C.c_uint, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.orc_kull_leibler.argtypes = [_u64p, C.c_uint]
    L.orc_kull_leibler.restype = C.c_double
    L.orc_update_trivial_gpu.argtypes = [_u64p, C.c_uint, _f64p]
    L.orc_update_trivial_cpu.argtypes = [_u64p, C.c_uint, _f64p]
    L.orc_weight_recursion.argtypes = [_u64p, C.c_uint, _f64p, C.c_int, C.c_int, _f64p]
    L.orc_flatness.argtypes = [_u64p, C.c_uint, C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.orc_jackknife.argtypes = [_f64p, C.c_uint, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.orc_weight_shift.argtypes = [C.c_double, C.c_double, C.c_uint, _f64p]
    L.orc_boltz.argtypes = [C.c_double, C.c_double, C.c_uint, _f64p, _f64p, C.c_int]
    L.orc_observables.argtypes = [C.c_double, C.c_uint, _u64p, _f64p, _f64p]
    L.orc_weight_run.argtypes = [C.POINTER(WeightOpts), _i8p, _i32p, _i32p, _f64p, _f64p, _f64p,
                                 C.c_uint, C.POINTER(C.c_int)]
    L.orc_weight_run.restype = C.c_uint
    L.orc_set_logf_table.argtypes = [C.c_void_p]
    L.orc_libm_logf_table.argtypes = [_f32p]
    L.orc_set_beta.argtypes = [C.c_double]
    _LIB = L
    return L


# --------------------------------------------------------------------------
# The device's acceptance logarithm (devlogf.cu)

_LOGF_TAB = None


def device_logf_table(device: int = 0) -> np.ndarray:
    """CUDA's logf((2k+1) 2^-24) for k < 2^23, evaluated on `device` (needs a
    GPU and oracle/_build/libdevlogf.so from build(refgpu=True))."""
    global _LOGF_TAB
    if _LOGF_TAB is None:
        path = os.path.join(BUILD, "libdevlogf.so")
        if not os.path.exists(path):
            build(refgpu=True)
        D = C.CDLL(path)
        D.orc_device_logf_table.argtypes = [C.c_int, _f32p, C.c_char_p, C.c_int]
        tab = np.empty(1 << 23, np.float32)
        err = C.create_string_buffer(256)
        if D.orc_device_logf_table(device, tab, err, 256) != 0:
            raise RuntimeError("device logf table: " + err.value.decode())
        _LOGF_TAB = tab
    return _LOGF_TAB


def use_device_logf(on: bool = True) -> None:
    """Make the oracle's weight and production sweeps decide with the device's
    logf (on) or with libm's (off)."""
    lib().orc_set_logf_table(device_logf_table().ctypes.data if on else None)


# --------------------------------------------------------------------------
# Convenience wrappers (numpy in / numpy out)

def philox(ctr, key, rounds=7):
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32(rounds, np.asarray(ctr, np.uint32), np.asarray(key, np.uint32), out)
    return out


def tables(L):
    N = L * L
    nv = np.zeros(4 * N, np.uint32)
    ix = np.zeros(N, np.uint32)
    lib().orc_sweep_tables(L, nv, ix)
    return nv, ix


def init_lattice(L, nchains, scheme, chain0=0):
    lat = np.zeros(nchains * L * L, np.int8)
    lib().orc_init_lattice(L, chain0, nchains, C.byref(scheme), lat)
    return lat.reshape(nchains, L * L)


def init_lattice_graded(L, nchains, scheme, cpd, chain0=0):
    """The graded initial spins (an extension): worker W of cpd nonzero with
    probability (2W+1)/(2 cpd), from the same Philox words as init_lattice."""
    lat = np.zeros(nchains * L * L, np.int8)
    lib().orc_init_lattice_graded(L, chain0, nchains, cpd, C.byref(scheme), lat)
    return lat.reshape(nchains, L * L)


def scheme_weight(jack=0, gpu=0):
    return lib().orc_scheme_weight(jack, gpu)


def scheme_produce(gpu=0):
    return lib().orc_scheme_produce(gpu)


def scheme_muca_mag(jack=0):
    return lib().orc_scheme_muca_mag(jack)


def energies(L, lat):
    lat = np.ascontiguousarray(lat, np.int8)
    n = lat.shape[0]
    ej = np.zeros(n, np.int32)
    ed = np.zeros(n, np.int32)
    mg = np.zeros(n, np.int32)
    lib().orc_chain_energies(L, n, lat.reshape(-1), ej, ed, mg)
    return ej, ed, mg


def weight_sweep(L, lat, ej, edel, w32, iter_, seed, therm, nup, chain0=0, rounds=7, nthreads=1, hist=None):
    lat = np.ascontiguousarray(lat, np.int8)
    n = lat.shape[0]
    N = L * L
    h = np.zeros(N + 1, np.uint64) if hist is None else hist
    flat = lat.reshape(-1)
    lib().orc_weight_sweep(L, chain0, n, flat, ej, edel, np.ascontiguousarray(w32, np.float32), h,
                           iter_, seed, therm, nup, rounds, nthreads)
    return flat.reshape(n, N), h


def produce_sweep(L, lat, ej, edel, mag, w64, iter_, seed, therm, nup, chain0=0, rounds=7, nthreads=1, hist=None):
    lat = np.ascontiguousarray(lat, np.int8)
    n = lat.shape[0]
    N = L * L
    h = np.zeros((N + 1) * (N + 2) // 2, np.uint64) if hist is None else hist
    flat = lat.reshape(-1)
    lib().orc_produce_sweep(L, chain0, n, flat, ej, edel, mag, np.ascontiguousarray(w64, np.float64), h,
                            iter_, seed, therm, nup, rounds, nthreads)
    return flat.reshape(n, N), h


def hist_range(h):
    s, e = C.c_int(), C.c_int()
    lib().orc_hist_range(np.ascontiguousarray(h, np.uint64), len(h) - 1, C.byref(s), C.byref(e))
    return s.value, e.value


def kull_leibler(h):
    return lib().orc_kull_leibler(np.ascontiguousarray(h, np.uint64), len(h) - 1)


def flatness(h):
    m, s, e = C.c_double(), C.c_int(), C.c_int()
    lib().orc_flatness(np.ascontiguousarray(h, np.uint64), len(h) - 1, C.byref(m), C.byref(s), C.byref(e))
    return m.value


def jackknife(x):
    a, e = C.c_double(), C.c_double()
    x = np.ascontiguousarray(x, np.float64)
    lib().orc_jackknife(x, len(x), C.byref(a), C.byref(e))
    return a.value, e.value


def observables(beta, N, hist2d, boltz):
    out = np.zeros(7)
    lib().orc_observables(beta, N, np.ascontiguousarray(hist2d, np.uint64), np.ascontiguousarray(boltz), out)
    return out


# --------------------------------------------------------------------------
# Reference harness (present only where the reference checkout was built)

_REF = None
_GH = None
_RG = None


def reflib():
    global _REF
    if _REF is not None:
        return _REF or None
    path = os.path.join(REFOUT, "libref_cpu.so")
    if not os.path.exists(path):
        _REF = False
        return None
    R = C.CDLL(path)
    ulp = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
    R.refp_mcs.argtypes = [C.c_uint, C.c_uint, _i32p, ulp, _f64p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                           C.POINTER(C.c_int), C.c_uint, C.c_uint, C.c_ulonglong, C.c_ulonglong, _i32p, _i32p]
    R.refp_observables.argtypes = [C.c_double, C.c_double, C.c_uint, ulp, _f64p, _f64p, _f64p, _f64p, C.c_uint]
    R.refp_jakknife.argtypes = [_f64p, _f64p, _f64p, C.c_int, C.c_uint]
    R.refp_weight_shift.argtypes = [C.c_double, C.c_double, C.c_uint, _f64p]
    R.refp_total_energy.argtypes = [C.c_uint, _i32p]
    R.refp_total_energy.restype = C.c_int
    R.refm_mcs.argtypes = [C.c_uint, C.c_uint, _i32p, ulp, _f64p, _i32p, _i32p, C.POINTER(C.c_int),
                           C.POINTER(C.c_int), C.c_uint, C.c_uint, C.c_ulonglong, C.c_ulonglong]
    R.refm_hist_range.argtypes = [C.c_uint, ulp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    R.refm_kull_leiber.argtypes = [C.c_uint, ulp]
    R.refm_kull_leiber.restype = C.c_double
    R.refm_weight_recursion.argtypes = [C.c_uint, ulp, _f64p, C.c_int, C.c_int, _f64p]
    _REF = R
    return R


def gpuhost():
    global _GH
    if _GH is not None:
        return _GH or None
    path = os.path.join(REFOUT, "libref_gpuhost.so")
    if not os.path.exists(path):
        _GH = False
        return None
    G = C.CDLL(path)
    G.refg_hist_range.argtypes = [_u64p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    G.refg_kull_leibler.argtypes = [_u64p, C.c_int]
    G.refg_kull_leibler.restype = C.c_double
    G.refg_weight_recursion.argtypes = [C.c_uint, _u64p, _f64p, C.c_int, C.c_int, _f64p]
    G.refg_jakknife.argtypes = [_f64p, _f64p, _f64p, C.c_uint]
    G.refg_weight_shift.argtypes = [C.c_double, C.c_double, C.c_uint, _f64p]
    G.refg_observables.argtypes = [C.c_double, C.c_double, C.c_uint, _u64p, _f64p, _f64p, _f64p, _f64p, C.c_uint]
    G.refg_jakknife_range.argtypes = [_f64p, _f64p, _f64p, C.c_int, C.c_uint]
    _GH = G
    return G


def refgpu():
    """Launcher of the reference kernels; None where it or the cubins are absent."""
    global _RG
    if _RG is not None:
        return _RG or None
    path = os.path.join(BUILD, "librefgpu.so")
    if not (os.path.exists(path) and os.path.exists(REF_WEIGHT_CUBIN)):
        _RG = False
        return None
    G = C.CDLL(path)
    fp = C.POINTER(C.c_float)
    G.refgpu_weight_mcs.argtypes = [C.c_char_p, C.c_uint, C.c_uint, _i8p, _u32p, _f32p, _i32p, _i32p,
                                    C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_int, fp]
    G.refgpu_produce_mcs.argtypes = [C.c_char_p, C.c_uint, C.c_uint, _i8p, _u64p, _f64p, _i32p, _i32p, _i32p,
                                     C.c_uint, C.c_uint, C.c_ulonglong, C.c_ulonglong, C.c_int, fp]
    G.refgpu_last_error.restype = C.c_char_p
    _RG = G
    return G


def refgpu_weight(L, lat_chain_major, w32, ej, edel, iter_, seed, therm, nup, compute_energies=False):
    """Run the reference weight kernel on [chain][site] input; returns
    (lattice [chain][site], hist u64, ej, edel, ms)."""
    G = refgpu()
    n, N = lat_chain_major.shape
    sm = np.ascontiguousarray(lat_chain_major.T, np.int8).reshape(-1)
    h = np.zeros(N + 1, np.uint32)
    ej = np.ascontiguousarray(ej, np.int32).copy()
    ed = np.ascontiguousarray(edel, np.int32).copy()
    ms = C.c_float()
    rc = G.refgpu_weight_mcs(REF_WEIGHT_CUBIN.encode(), L, n, sm, h, np.ascontiguousarray(w32, np.float32),
                             ej, ed, iter_, seed, therm, nup, int(compute_energies), C.byref(ms))
    if rc != 0:
        raise RuntimeError("reference weight kernel failed: %s" % G.refgpu_last_error().decode())
    return sm.reshape(N, n).T.copy(), h.astype(np.uint64), ej, ed, ms.value


def refgpu_produce(L, lat_chain_major, w64, ej, edel, mag, iter_, seed, therm, nup, compute_energies=False):
    G = refgpu()
    n, N = lat_chain_major.shape
    sm = np.ascontiguousarray(lat_chain_major.T, np.int8).reshape(-1)
    h = np.zeros((N + 1) * (N + 2) // 2, np.uint64)
    ej = np.ascontiguousarray(ej, np.int32).copy()
    ed = np.ascontiguousarray(edel, np.int32).copy()
    mg = np.ascontiguousarray(mag, np.int32).copy()
    ms = C.c_float()
    rc = G.refgpu_produce_mcs(REF_PRODUCE_CUBIN.encode(), L, n, sm, h, np.ascontiguousarray(w64, np.float64),
                              ej, ed, mg, iter_, seed, therm, nup, int(compute_energies), C.byref(ms))
    if rc != 0:
        raise RuntimeError("reference production kernel failed: %s" % G.refgpu_last_error().decode())
    return sm.reshape(N, n).T.copy(), h, ej, ed, mg, ms.value
