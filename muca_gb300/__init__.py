"""muca_gb300 -- GB300-native multicanonical (MUCA) engine for the 2D
Blume-Capel model.

This module is a thin ctypes binding of the C ABI in include/muca.h, which is
implemented by hand-written sm_103a CUDA kernels in muca_gb300/csrc and built
into muca_gb300/_build/libmuca.so.  There is no CPU fallback: if the library
is missing or no GPU is present the calls raise.

The drop-in replacements for the reference programs multigpu_weight and
produce_gpu are the executables muca_gb300/_build/{multigpu_weight,produce_gpu}
(same positional command line, same output files).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmuca.so")

MODE_WEIGHT, MODE_PRODUCE = 0, 1
INIT_WEIGHT, INIT_PRODUCE, INIT_CHAIN_COUNTER, INIT_ORDERED, INIT_MUCA_MAG, INIT_GRADED = 0, 1, 2, 3, 4, 5
ALGO_SWEEP, ALGO_RANDOM_SITE = 0, 1
UPDATE_TRIVIAL, UPDATE_TRIVIAL_CPU, UPDATE_RECURSION = 0, 1, 2
KERNEL_AUTO, KERNEL_GENERIC, KERNEL_WINDOWED, KERNEL_SPECIALIZED = 0, 1, 2, 3
HOOK_SILENT_PRODUCER = 1
HOOK_FLUSH_ROWS = 2
STATUS = {0: "OK", 1: "BAD_ARG", 2: "CUDA", 3: "TIMEOUT", 4: "NOT_CONVERGED", 5: "IO", 6: "STATE"}

# Every symbol include/muca.h declares (the C-ABI surface).
EXPORTS = [
    "muca_create", "muca_destroy", "muca_last_error", "muca_get_info", "muca_default_chains",
    "muca_set_log_bracket", "muca_set_wait_limit", "muca_set_test_hooks",
    "muca_init_chains", "muca_set_lattice", "muca_get_lattice", "muca_get_chain_state",
    "muca_set_weights", "muca_get_weights", "muca_sweep", "muca_sweep_accumulate",
    "muca_clear_histogram", "muca_get_histogram", "muca_set_histogram", "muca_histogram_stats", "muca_update_weights",
    "muca_iterate_host",
    "muca_weight_run", "muca_weight_shift", "muca_compute_observables", "muca_jackknife",
    "muca_philox_peak", "muca_sweep_floor", "muca_weight_run_stream", "muca_get_reweighting_weights",
    "muca_observables_noalloc",
    "muca_batch_create", "muca_batch_destroy", "muca_batch_last_error", "muca_batch_get_info",
    "muca_batch_init_chains", "muca_batch_set_weights", "muca_batch_get_weights", "muca_batch_get_histogram",
    "muca_batch_run",
    "muca_mlp_param_count", "muca_mlp_create", "muca_mlp_destroy", "muca_mlp_last_error", "muca_mlp_get_params",
    "muca_mlp_set_params", "muca_mlp_set_data", "muca_mlp_train", "muca_mlp_grad", "muca_mlp_predict",
    "muca_mlp_log_weights",
]


class MucaError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class Params(C.Structure):
    _fields_ = [("L", C.c_uint32), ("nchains", C.c_uint32), ("ndev", C.c_uint32), ("device", C.c_int32),
                ("rounds", C.c_uint32), ("mode", C.c_uint32), ("stream", C.c_void_p), ("dev_offset", C.c_uint32),
                ("kernel", C.c_uint32), ("algorithm", C.c_uint32), ("host_logf", C.c_uint32)]


class Info(C.Structure):
    _fields_ = [("L", C.c_uint32), ("N", C.c_uint32), ("nchains_total", C.c_uint32),
                ("chains_per_block", C.c_uint32), ("blocks", C.c_uint32), ("lattice_in_smem", C.c_uint32),
                ("hist_in_smem", C.c_uint32), ("smem_bytes", C.c_uint32), ("sms", C.c_uint32),
                ("weights_in_smem", C.c_uint32), ("device_bytes", C.c_uint64), ("log_bracket", C.c_double),
                ("kernel", C.c_uint32), ("threads_per_block", C.c_uint32)]


class HistStats(C.Structure):
    _fields_ = [("start", C.c_int32), ("end", C.c_int32), ("width", C.c_uint32), ("visited", C.c_uint32),
                ("events", C.c_uint64), ("min_count", C.c_uint64), ("d_kl", C.c_double),
                ("min_over_mean", C.c_double)]


class RunOpts(C.Structure):
    _fields_ = [("jack", C.c_uint32), ("starting_M", C.c_uint32), ("therm", C.c_uint32), ("rule", C.c_uint32),
                ("hold_until_full", C.c_uint32), ("flat_minmean", C.c_uint32), ("max_iter", C.c_uint32),
                ("init_scheme", C.c_uint32), ("reinit_chains", C.c_uint32), ("nup_schedule", C.c_uint32),
                ("min_over_mean", C.c_double), ("d_kl_max", C.c_double), ("width_start", C.c_uint32),
                ("nup_max", C.c_uint32), ("graph_iters", C.c_uint32)]


class IterRecord(C.Structure):
    _fields_ = [("k", C.c_uint32), ("width_temp", C.c_uint32), ("width", C.c_uint32), ("nupdates", C.c_uint32),
                ("total_run", C.c_uint64), ("d_kl", C.c_double), ("min_over_mean", C.c_double),
                ("kernel_ms", C.c_double), ("memcpy_ms", C.c_double)]


ITER_CB = None  # set below, after IterRecord


class RunResult(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("converged", C.c_uint32), ("width_reached_iter", C.c_uint32),
                ("total_run", C.c_uint64), ("nwidth_step", C.c_uint64), ("total_kernel_s", C.c_double),
                ("total_mem_s", C.c_double), ("nwidth_time_s", C.c_double), ("wall_s", C.c_double)]


ITER_CB = C.CFUNCTYPE(None, C.POINTER(IterRecord), C.c_void_p)


class Instance(C.Structure):
    _fields_ = [("L", C.c_uint32), ("nchains", C.c_uint32), ("seed", C.c_uint32), ("reserved", C.c_uint32),
                ("beta", C.c_double)]


class BatchShape(C.Structure):
    _fields_ = [("chains_per_block", C.c_uint32), ("lattice_in_smem", C.c_uint32), ("hist_in_smem", C.c_uint32),
                ("blocks_per_sm", C.c_uint32), ("ms", C.c_double)]


class BatchParams(C.Structure):
    _fields_ = [("device", C.c_int32), ("rounds", C.c_uint32), ("stream", C.c_void_p),
                ("shape_chains_per_block", C.c_uint32), ("shape_lattice_in_smem", C.c_uint32),
                ("shape_hist_in_smem", C.c_uint32)]


class BatchInfo(C.Structure):
    _fields_ = [("n_instances", C.c_uint32), ("n_items", C.c_uint32), ("grid", C.c_uint32), ("threads", C.c_uint32),
                ("smem_bytes", C.c_uint32), ("n_tried", C.c_uint32), ("shape", BatchShape),
                ("tried", BatchShape * 32), ("device_bytes", C.c_uint64), ("log_bracket", C.c_double)]


class BatchRunOpts(C.Structure):
    _fields_ = [("starting_M", C.c_uint32), ("rule", C.c_uint32), ("nup_schedule", C.c_uint32),
                ("flat_minmean", C.c_uint32), ("max_iter", C.c_uint32), ("graph_iters", C.c_uint32),
                ("reinit_chains", C.c_uint32), ("nup_max", C.c_uint32), ("min_over_mean", C.c_double),
                ("d_kl_max", C.c_double), ("starting_sweeps", C.c_uint32), ("graded_init", C.c_uint32)]


class BatchResult(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("converged", C.c_uint32), ("width", C.c_uint32),
                ("reach_iter", C.c_uint32), ("nupdates", C.c_uint32), ("reserved", C.c_uint32),
                ("total_run", C.c_uint64), ("d_kl", C.c_double), ("min_over_mean", C.c_double)]


class Observables(C.Structure):
    _fields_ = [("m_abs", C.c_double), ("chi", C.c_double), ("u4", C.c_double), ("sum", C.c_double),
                ("m1", C.c_double), ("m2", C.c_double), ("m4", C.c_double)]


_LIB = None


def lib():
    """Load libmuca.so (raises if it was not built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise ImportError("muca_gb300: %s is missing; run `python -c 'import __graft_entry__ as g; g.build()'`"
                          % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    i8 = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")
    i32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    u64 = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
    f64 = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    L.muca_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
    L.muca_destroy.argtypes = [vp]
    L.muca_last_error.argtypes = [vp]
    L.muca_last_error.restype = C.c_char_p
    L.muca_get_info.argtypes = [vp, C.POINTER(Info)]
    L.muca_default_chains.argtypes = [C.c_int32, C.POINTER(C.c_uint32)]
    L.muca_set_log_bracket.argtypes = [vp, C.c_double]
    L.muca_set_wait_limit.argtypes = [vp, C.c_uint64]
    L.muca_set_test_hooks.argtypes = [vp, C.c_uint32]
    L.muca_init_chains.argtypes = [vp, C.c_uint32, C.c_uint32]
    L.muca_set_lattice.argtypes = [vp, i8, C.c_size_t]
    L.muca_get_lattice.argtypes = [vp, i8, C.c_size_t]
    L.muca_get_chain_state.argtypes = [vp, i32, i32, i32, C.c_size_t]
    L.muca_set_weights.argtypes = [vp, f64, C.c_size_t]
    L.muca_get_weights.argtypes = [vp, f64, C.c_size_t]
    L.muca_sweep.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint64]
    L.muca_sweep_accumulate.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint64]
    L.muca_clear_histogram.argtypes = [vp]
    L.muca_get_histogram.argtypes = [vp, u64, C.c_size_t]
    L.muca_set_histogram.argtypes = [vp, u64, C.c_size_t]
    L.muca_histogram_stats.argtypes = [vp, C.POINTER(HistStats)]
    L.muca_update_weights.argtypes = [vp, C.c_uint32, C.POINTER(HistStats)]
    L.muca_iterate_host.argtypes = [vp, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint64,
                                    C.c_uint32, C.c_void_p, C.c_void_p, C.POINTER(HistStats)]
    L.muca_weight_run.argtypes = [vp, C.POINTER(RunOpts), C.POINTER(RunResult), C.POINTER(IterRecord), C.c_size_t]
    L.muca_weight_shift.argtypes = [vp, C.c_double, C.c_double]
    L.muca_get_reweighting_weights.argtypes = [vp, f64, C.c_size_t]
    L.muca_weight_run_stream.argtypes = [vp, C.POINTER(RunOpts), C.POINTER(RunResult), ITER_CB, C.c_void_p]
    L.muca_compute_observables.argtypes = [vp, C.c_double, C.c_double, C.POINTER(Observables)]
    L.muca_jackknife.argtypes = [vp, f64, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.muca_philox_peak.argtypes = [C.c_int32, C.c_uint32, C.POINTER(C.c_double)]
    L.muca_sweep_floor.argtypes = [C.c_int32, C.c_uint32, C.c_uint32, C.POINTER(C.c_double)]
    L.muca_observables_noalloc.argtypes = [C.c_int32, vp, vp, C.c_uint32, C.c_double, C.c_double, vp, vp]
    L.muca_batch_create.argtypes = [C.POINTER(BatchParams), C.POINTER(Instance), C.c_uint32, C.POINTER(vp)]
    L.muca_batch_destroy.argtypes = [vp]
    L.muca_batch_last_error.argtypes = [vp]
    L.muca_batch_last_error.restype = C.c_char_p
    L.muca_batch_get_info.argtypes = [vp, C.POINTER(BatchInfo)]
    L.muca_batch_init_chains.argtypes = [vp]
    L.muca_batch_set_weights.argtypes = [vp, C.c_uint32, f64, C.c_size_t]
    L.muca_batch_get_weights.argtypes = [vp, C.c_uint32, f64, C.c_size_t]
    L.muca_batch_get_histogram.argtypes = [vp, C.c_uint32, u64, C.c_size_t]
    L.muca_batch_run.argtypes = [vp, C.POINTER(BatchRunOpts), C.POINTER(BatchResult), C.POINTER(C.c_double)]
    f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    L.muca_mlp_param_count.restype = C.c_size_t
    L.muca_mlp_create.argtypes = [C.c_int32, C.c_uint64, vp, C.POINTER(vp)]
    L.muca_mlp_destroy.argtypes = [vp]
    L.muca_mlp_last_error.argtypes = [vp]
    L.muca_mlp_last_error.restype = C.c_char_p
    L.muca_mlp_get_params.argtypes = [vp, f32, C.c_size_t]
    L.muca_mlp_set_params.argtypes = [vp, f32, C.c_size_t]
    L.muca_mlp_set_data.argtypes = [vp, f32, f32, C.c_uint32]
    L.muca_mlp_train.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_float, C.c_uint32, vp]
    L.muca_mlp_grad.argtypes = [vp, f32, f32, C.c_uint32, f32, C.POINTER(C.c_float)]
    L.muca_mlp_predict.argtypes = [vp, f32, C.c_uint32, f32]
    L.muca_mlp_log_weights.argtypes = [vp, C.c_uint32, C.c_double, C.c_double, f64, C.c_size_t]
    _LIB = L
    return L


def philox_peak(device: int = 0, rounds: int = 7) -> float:
    """Measured Philox4x32-R blocks per second on this GPU (integer-pipe ceiling)."""
    out = C.c_double()
    st = lib().muca_philox_peak(device, rounds, C.byref(out))
    if st:
        raise MucaError(st, lib().muca_last_error(None).decode())
    return out.value


SWEEP_FLOOR_PARTS = ("whole_window", "draws_and_decode", "scan_store_histogram", "decision_chain", "draws",
                     "fp32_add_latency", "shared_load_latency")


def sweep_floor(part: int, device: int = 0, windows: int = 4096) -> float:
    """SM cycles per attempt of one warp for a part of the weight-mode
    windowed sweep at L = 72 (muca_sweep_floor): 0 the whole window, 1 draws
    and decode, 2 scan, store and histogram, 3 the bare decision chain, 4 the
    draws; 5 and 6 the latency of one dependent FP32 add and of one
    dependent shared-memory load."""
    out = C.c_double()
    st = lib().muca_sweep_floor(device, part, windows, C.byref(out))
    if st:
        raise MucaError(st, lib().muca_last_error(None).decode())
    return out.value


def observables_noalloc(device, d_hist2d, d_lnw, L, beta, delta, d_sums, stream=None) -> None:
    """muca_observables_noalloc on raw device addresses (ints): the four
    reweighting sums into d_sums, enqueued on `stream` (a cudaStream_t as int,
    None = the legacy default stream); nothing is allocated."""
    st = lib().muca_observables_noalloc(device, d_hist2d, d_lnw, L, beta, delta, d_sums, stream)
    if st:
        raise MucaError(st, lib().muca_last_error(None).decode())


def default_chains(device: int = 0) -> int:
    out = C.c_uint32()
    st = lib().muca_default_chains(device, C.byref(out))
    if st:
        raise MucaError(st, lib().muca_last_error(None).decode())
    return out.value


class Engine:
    """One simulation context (all chains of one lattice size) on one GPU."""

    def __init__(self, L, nchains=0, ndev=1, mode=MODE_WEIGHT, rounds=7, device=0, stream=None, dev_offset=0,
                 kernel=KERNEL_AUTO, algorithm=ALGO_SWEEP, host_logf=0):
        self._lib = lib()
        p = Params(L=L, nchains=nchains, ndev=ndev, device=device, rounds=rounds, mode=mode,
                   stream=C.c_void_p(stream) if stream else None, dev_offset=dev_offset, kernel=kernel,
                   algorithm=algorithm, host_logf=host_logf)
        h = C.c_void_p()
        st = self._lib.muca_create(C.byref(p), C.byref(h))
        if st:
            raise MucaError(st, self._lib.muca_last_error(None).decode())
        self._h = h
        self.L, self.N, self.mode = L, L * L, mode
        self.info = self._info()
        self.nchains = self.info.nchains_total

    # -- plumbing --------------------------------------------------------
    def _ck(self, st):
        if st:
            raise MucaError(st, self._lib.muca_last_error(self._h).decode())

    def _info(self):
        i = Info()
        self._ck(self._lib.muca_get_info(self._h, C.byref(i)))
        return i

    def close(self):
        if getattr(self, "_h", None):
            self._lib.muca_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- chains / weights --------------------------------------------------
    def init_chains(self, scheme=INIT_WEIGHT, jack=0):
        self._ck(self._lib.muca_init_chains(self._h, scheme, jack))

    def set_lattice(self, lat):
        a = np.ascontiguousarray(lat, np.int8).reshape(-1)
        self._ck(self._lib.muca_set_lattice(self._h, a, a.size))

    def get_lattice(self):
        a = np.zeros(self.nchains * self.N, np.int8)
        self._ck(self._lib.muca_get_lattice(self._h, a, a.size))
        return a.reshape(self.nchains, self.N)

    def chain_state(self):
        ej = np.zeros(self.nchains, np.int32)
        ed = np.zeros(self.nchains, np.int32)
        mg = np.zeros(self.nchains, np.int32)
        self._ck(self._lib.muca_get_chain_state(self._h, ej, ed, mg, self.nchains))
        return ej, ed, mg

    def set_weights(self, lnw):
        a = np.ascontiguousarray(lnw, np.float64)
        self._ck(self._lib.muca_set_weights(self._h, a, a.size))

    def get_weights(self, out=None):
        a = np.zeros(self.N + 1) if out is None else out
        self._ck(self._lib.muca_get_weights(self._h, a, a.size))
        return a

    # -- sweeps ----------------------------------------------------------
    def sweep(self, iter_, seed_base, seed_dev_mul, therm, nup, accumulate=False):
        f = self._lib.muca_sweep_accumulate if accumulate else self._lib.muca_sweep
        self._ck(f(self._h, iter_, seed_base, seed_dev_mul, therm, nup))

    def set_log_bracket(self, bracket):
        """Widen the fast acceptance test's bound (1e30: every window takes
        the exact replay)."""
        self._ck(self._lib.muca_set_log_bracket(self._h, float(bracket)))

    def set_wait_limit(self, cycles):
        """Bound of every device-side wait of the warp-specialised sweep, in
        SM clock cycles without progress (0 = the default, about 8 s)."""
        self._ck(self._lib.muca_set_wait_limit(self._h, int(cycles)))

    def set_test_hooks(self, hooks):
        """Test hooks (HOOK_SILENT_PRODUCER, HOOK_FLUSH_ROWS); 0 = none."""
        self._ck(self._lib.muca_set_test_hooks(self._h, int(hooks)))

    def clear_histogram(self):
        self._ck(self._lib.muca_clear_histogram(self._h))

    def histogram(self, out=None):
        n = self.N + 1 if self.mode == MODE_WEIGHT else (self.N + 1) * (self.N + 2) // 2
        h = np.zeros(n, np.uint64) if out is None else out
        self._ck(self._lib.muca_get_histogram(self._h, h, n))
        return h

    def set_histogram(self, h):
        a = np.ascontiguousarray(h, np.uint64)
        self._ck(self._lib.muca_set_histogram(self._h, a, a.size))

    def hist_stats(self):
        s = HistStats()
        self._ck(self._lib.muca_histogram_stats(self._h, C.byref(s)))
        return s

    def update_weights(self, rule=UPDATE_TRIVIAL, wait=True):
        """FP64 weight update on the device; wait=False only enqueues it."""
        if not wait:
            self._ck(self._lib.muca_update_weights(self._h, rule, None))
            return None
        s = HistStats()
        self._ck(self._lib.muca_update_weights(self._h, rule, C.byref(s)))
        return s

    def iterate_host(self, lnw_in, iter, seed_base, seed_dev_mul, therm, nup, rule=UPDATE_TRIVIAL, lnw_out=None,
                     hist_out=None, stats=False):
        """One weight iteration with host buffers and one synchronisation:
        weights in (None keeps the device's), sweep, update, then the updated
        weights and the histogram into the given float64 / uint64 arrays of
        N+1 (either may be None).  Returns the histogram summary if stats."""
        n = self.N + 1

        def arr(a, dt):
            if a is None:
                return None
            if a.dtype != dt or a.size != n or not a.flags.c_contiguous:
                raise ValueError("expected a contiguous %s array of %d values" % (dt, n))
            return a.ctypes.data
        s = HistStats() if stats else None
        self._ck(self._lib.muca_iterate_host(self._h, arr(lnw_in, np.float64), iter, seed_base, seed_dev_mul,
                                             therm, nup, rule, arr(lnw_out, np.float64),
                                             arr(hist_out, np.uint64), C.byref(s) if stats else None))
        return s

    def weight_run(self, starting_M=1, jack=0, rule=UPDATE_TRIVIAL, hold_until_full=0, flat_minmean=0,
                   max_iter=0, therm=0, init_scheme=INIT_WEIGHT, reinit_chains=1, nup_schedule=0,
                   min_over_mean=0.0, d_kl_max=0.0, width_start=0, nup_max=0, records=1000, graph_iters=0,
                   raise_on_not_converged=False):
        o = RunOpts(jack=jack, starting_M=starting_M, therm=therm, rule=rule, hold_until_full=hold_until_full,
                    flat_minmean=flat_minmean, max_iter=max_iter, init_scheme=init_scheme,
                    reinit_chains=reinit_chains, nup_schedule=nup_schedule, min_over_mean=min_over_mean,
                    d_kl_max=d_kl_max, width_start=width_start, nup_max=nup_max, graph_iters=graph_iters)
        res = RunResult()
        recs = (IterRecord * max(records, 1))()
        st = self._lib.muca_weight_run(self._h, C.byref(o), C.byref(res), recs, records)
        if st and (st != 4 or raise_on_not_converged):
            self._ck(st)
        n = min(res.iterations, records)
        return res, [recs[i] for i in range(n)]

    # -- production --------------------------------------------------------
    def weight_shift(self, beta, delta):
        self._ck(self._lib.muca_weight_shift(self._h, beta, delta))

    def reweighting_weights(self):
        a = np.zeros(self.N + 1)
        self._ck(self._lib.muca_get_reweighting_weights(self._h, a, a.size))
        return a

    def observables(self, beta, delta):
        o = Observables()
        self._ck(self._lib.muca_compute_observables(self._h, beta, delta, C.byref(o)))
        return o

    def jackknife(self, x):
        x = np.ascontiguousarray(x, np.float64)
        a, e = C.c_double(), C.c_double()
        self._ck(self._lib.muca_jackknife(self._h, x, x.size, C.byref(a), C.byref(e)))
        return a.value, e.value



class Batch:
    """Many independent weight runs of uneven size on one GPU (muca_batch_*).

    instances: sequence of (L, nchains, beta, seed).  shape: None (autotune)
    or (chains_per_block, lattice_in_smem, hist_in_smem)."""

    def __init__(self, instances, device=0, rounds=7, stream=None, shape=None):
        self._lib = lib()
        self.instances = [tuple(x) for x in instances]
        arr = (Instance * len(self.instances))()
        for k, (L, nc, beta, seed) in enumerate(self.instances):
            arr[k] = Instance(L=L, nchains=nc, seed=seed, reserved=0, beta=beta)
        p = BatchParams(device=device, rounds=rounds, stream=C.c_void_p(stream) if stream else None)
        if shape is not None:
            p.shape_chains_per_block, p.shape_lattice_in_smem, p.shape_hist_in_smem = shape
        h = C.c_void_p()
        st = self._lib.muca_batch_create(C.byref(p), arr, len(self.instances), C.byref(h))
        if st:
            raise MucaError(st, self._lib.muca_batch_last_error(None).decode())
        self._h = h

    def _ck(self, st, allow=()):
        if st and st not in allow:
            raise MucaError(st, self._lib.muca_batch_last_error(self._h).decode())
        return st

    def close(self):
        if getattr(self, "_h", None):
            self._lib.muca_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self):
        o = BatchInfo()
        self._ck(self._lib.muca_batch_get_info(self._h, C.byref(o)))
        return o

    def init_chains(self):
        self._ck(self._lib.muca_batch_init_chains(self._h))

    def set_weights(self, i, lnw):
        a = np.ascontiguousarray(lnw, np.float64)
        self._ck(self._lib.muca_batch_set_weights(self._h, i, a, a.size))

    def get_weights(self, i):
        L = self.instances[i][0]
        a = np.zeros(L * L + 1)
        self._ck(self._lib.muca_batch_get_weights(self._h, i, a, a.size))
        return a

    def histogram(self, i):
        L = self.instances[i][0]
        a = np.zeros(L * L + 1, np.uint64)
        self._ck(self._lib.muca_batch_get_histogram(self._h, i, a, a.size))
        return a

    def run(self, starting_M=1, rule=UPDATE_TRIVIAL, nup_schedule=0, flat_minmean=0, max_iter=0, graph_iters=0,
            reinit_chains=0, min_over_mean=0.0, d_kl_max=0.0, nup_max=0, starting_sweeps=0, graded_init=0,
            raise_on_not_converged=False):
        """Returns (list of BatchResult, device seconds)."""
        o = BatchRunOpts(starting_M=starting_M, rule=rule, nup_schedule=nup_schedule, flat_minmean=flat_minmean,
                         max_iter=max_iter, graph_iters=graph_iters, reinit_chains=reinit_chains, nup_max=nup_max,
                         min_over_mean=min_over_mean, d_kl_max=d_kl_max, starting_sweeps=starting_sweeps,
                         graded_init=graded_init)
        res = (BatchResult * len(self.instances))()
        sec = C.c_double()
        self._ck(self._lib.muca_batch_run(self._h, C.byref(o), res, C.byref(sec)),
                 allow=() if raise_on_not_converged else (4,))
        return list(res), sec.value



class MLP:
    """The warm-start network (muca_mlp_*): (L/128, T, Delta, E_Delta/N) ->
    (lnW - mean lnW)/N, 3 x 128 SiLU, FP32, trained on the device."""

    def __init__(self, device=0, seed=0, stream=None):
        self._lib = lib()
        h = C.c_void_p()
        st = self._lib.muca_mlp_create(device, seed, C.c_void_p(stream) if stream else None, C.byref(h))
        if st:
            raise MucaError(st, self._lib.muca_mlp_last_error(None).decode())
        self._h = h
        self.n_params = int(self._lib.muca_mlp_param_count())

    def _ck(self, st):
        if st:
            raise MucaError(st, self._lib.muca_mlp_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.muca_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def params(self):
        p = np.zeros(self.n_params, np.float32)
        self._ck(self._lib.muca_mlp_get_params(self._h, p, p.size))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self._ck(self._lib.muca_mlp_set_params(self._h, p, p.size))

    def set_data(self, x, t):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 4)
        t = np.ascontiguousarray(t, np.float32).reshape(-1)
        assert x.shape[0] == t.size
        self._ck(self._lib.muca_mlp_set_data(self._h, x, t, t.size))

    def train(self, steps, batch=4096, lr=1e-3, seed=0):
        losses = np.zeros(steps, np.float32)
        self._ck(self._lib.muca_mlp_train(self._h, steps, batch, lr, seed, losses.ctypes.data))
        return losses

    def grad(self, x, t):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 4)
        t = np.ascontiguousarray(t, np.float32).reshape(-1)
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_float()
        self._ck(self._lib.muca_mlp_grad(self._h, x, t, t.size, g, C.byref(loss)))
        return loss.value, g

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 4)
        y = np.zeros(x.shape[0], np.float32)
        self._ck(self._lib.muca_mlp_predict(self._h, x, x.shape[0], y))
        return y

    def log_weights(self, L, T, delta):
        w = np.zeros(L * L + 1)
        self._ck(self._lib.muca_mlp_log_weights(self._h, L, T, delta, w, w.size))
        return w


def mlp_features(L, T, delta, lnw):
    """Training pairs of one converged weight: x = (L/128, T, Delta, i/N),
    t = (lnW_i - mean lnW)/N for i = 0..N."""
    lnw = np.asarray(lnw, np.float64)
    N = lnw.size - 1
    x = np.zeros((N + 1, 4), np.float32)
    x[:, 0] = L / 128.0
    x[:, 1] = T
    x[:, 2] = delta
    x[:, 3] = np.arange(N + 1) / N
    t = ((lnw - lnw.mean()) / N).astype(np.float32)
    return x, t
