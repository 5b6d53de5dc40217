/*
 * muca.h -- C ABI of the GB300 multicanonical (MUCA) engine for the 2D
 * Blume-Capel model.
 *
 * The reference (null2p/MUCA) has no library interface: its boundary is the
 * command line and files of two CUDA programs, multigpu_weight
 * (muca_delta_multigpu.cu) and produce_gpu (produce2_multigpu.cu).  This ABI
 * is the layer underneath the drop-in executables of this project (which keep
 * that command line and those files); each entry point names the reference
 * code it replaces.  Plain pointers and sizes only: host buffers are owned by
 * the caller, device buffers by the context.
 *
 * Conventions
 *  - Every call returns a muca_status; muca_last_error() gives the text.
 *  - A context serves one host thread and one CUDA stream.  It is not
 *    thread-safe; separate contexts may be driven from separate threads.
 *  - Lattices cross the ABI as int8 [chain][site], site = row*L + col, spins
 *    in {-1, 0, +1}.  Chain c is the reference's WORKER c of emulated device
 *    c / nchains (the reference's starting_gpu..last_gpu range becomes
 *    `ndev` emulated devices on one GPU, each with its own seeds).
 *  - The multicanonical variable is E_Delta = sum_i s_i^2 in [0, N], N = L*L
 *    (muca_delta_multigpu.cu:195,810,823); weights and the weight-run
 *    histogram have N+1 entries.  The production histogram is over
 *    (E_Delta, M) packed at (M + E_Delta^2 + 2 E_Delta)/2, (N+1)(N+2)/2
 *    entries (produce2_multigpu.cu:489).
 *  - beta = 2 (T = 0.5) is fixed in the Metropolis step, as in the
 *    reference (muca_delta_multigpu.cu:810).
 */
#ifndef MUCA_H
#define MUCA_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MUCA_ABI_VERSION 1

typedef struct muca_ctx muca_ctx;

typedef enum muca_status {
    MUCA_OK = 0,
    MUCA_ERR_BAD_ARG = 1,       /* invalid argument (size, L, pointer, lattice value) */
    MUCA_ERR_CUDA = 2,          /* a CUDA call failed */
    MUCA_ERR_TIMEOUT = 3,       /* a bounded device loop gave up */
    MUCA_ERR_NOT_CONVERGED = 4, /* weight run hit max_iter */
    MUCA_ERR_IO = 5,            /* file read/write failed or malformed file */
    MUCA_ERR_STATE = 6          /* call not valid in the current context state */
} muca_status;

typedef enum muca_mode {
    MUCA_MODE_WEIGHT = 0,  /* FP32 weight shadow, 1D histogram of E_Delta (multigpu_weight) */
    MUCA_MODE_PRODUCE = 1  /* FP64 weights, M tracked, 2D (E_Delta, M) histogram (produce_gpu) */
} muca_mode;

typedef enum muca_init_scheme {
    MUCA_INIT_WEIGHT = 0,   /* muca_delta_multigpu.cu:340-351: key {10W+2*jack, 0xdecafbad},
                               ctr {2*dev, 100, 0xBADCAB1E, 0xBADC0DED}, ++ctr[0] per 4 sites */
    MUCA_INIT_PRODUCE = 1,  /* produce2_multigpu.cu:126-138: key {10W, 0xdecafbad},
                               ctr {1000*dev, 100, 0, 0xBADCAFE3}, ++ctr[2] per 4 sites */
    MUCA_INIT_CHAIN_COUNTER = 2, /* extension: Philox4x32-10, key {2024, jack}, ctr {chain, group, 0, 0} */
    MUCA_INIT_ORDERED = 3,  /* extension for rand_config=0: every spin +1 */
    MUCA_INIT_GRADED = 5,   /* extension: the Philox words of MUCA_INIT_WEIGHT, each spin nonzero with
                               probability (2W+1)/(2 nchains-per-device) (sign from the word's bit 0),
                               so the chains' E_Delta cover [0, N] evenly from the start */
    MUCA_INIT_MUCA_MAG = 4  /* muca_mag.cpp:63-73 (the CPU weight program): key {10W + 10000*jack,
                               0xdecafbad}, ctr {0, 100, 0xBADCAB1E, 0xBADC0DED}, ++ctr[0] per 4 sites */
} muca_init_scheme;

typedef enum muca_algorithm {
    MUCA_ALGO_SWEEP = 0,      /* the GPU programs' kernels: sites in sweep order, two Philox streams */
    MUCA_ALGO_RANDOM_SITE = 1 /* the CPU weight program's mcs (muca_mag.cpp:312-393) and its GPU port
                                 mcs2 (muca_delta_multigpu.cu:637-734): random site, three Philox
                                 streams, FP64 weights; weight mode only */
} muca_algorithm;

typedef enum muca_update_rule {
    MUCA_UPDATE_TRIVIAL = 0,     /* muca_delta_multigpu.cu:466-476: lnW -= ln H for H>1; lnW -= lnW[0] */
    MUCA_UPDATE_TRIVIAL_CPU = 1, /* muca_mag.cpp:178-183: H>0 variant, normalise bins with H>0 only */
    MUCA_UPDATE_RECURSION = 2    /* muca_delta_multigpu.cu:833-859 weight_recursion, then lnW -= lnW[0] */
} muca_update_rule;

typedef struct muca_params {
    uint32_t L;        /* lattice side, 2..128 */
    uint32_t nchains;  /* chains per emulated device (reference NUM_WORKERS);
                          0 = reference formula maxThreadsPerSM * SMs (muca_delta_multigpu.cu:100-106) */
    uint32_t ndev;     /* emulated devices (reference last_gpu-starting_gpu+1); 0 means 1 */
    int32_t device;    /* CUDA device ordinal */
    uint32_t rounds;   /* Philox4x32 rounds: 7 (reference, muca_delta_multigpu.cu:21) or 10; 0 means 7 */
    uint32_t mode;     /* muca_mode */
    void *stream;      /* cudaStream_t to launch on; NULL = the context creates one */
    uint32_t dev_offset; /* index of the first emulated device (a process that runs
                            reference devices k..k+ndev-1 sets k; seeds and init
                            counters follow the device index) */
    uint32_t kernel;     /* sweep kernel: 0 auto (windowed when L % 8 == 0, else generic),
                            1 generic (reference step by step), 2 windowed,
                            3 warp-specialised (2 and 3 need L % 8 == 0) */
    uint32_t algorithm;  /* muca_algorithm */
    uint32_t host_logf;  /* random-site algorithm: 1 = the acceptance log is the host libm's logf
                            (what the CPU program computes; bit-exact with it), 0 = CUDA's logf (mcs2) */
} muca_params;

typedef struct muca_info {
    uint32_t L, N, nchains_total, chains_per_block, blocks, lattice_in_smem, hist_in_smem;
    uint32_t smem_bytes, sms, weights_in_smem;
    uint64_t device_bytes;
    double log_bracket;  /* bound used by the fast acceptance test: twice the measured
                            max |__logf(u) - logf(u)| over all u01fixedpt<float> values */
    uint32_t kernel;      /* sweep kernel in use (see muca_params.kernel) */
    uint32_t threads_per_block;
} muca_info;

/* Histogram summary (muca_delta_multigpu.cu:431-447 and the min/mean test of
 * the flatness criterion): range of bins with H>1 (hist_range :573-596),
 * Kullback-Leibler divergence against uniform over visited bins (:598-618). */
typedef struct muca_hist_stats {
    int32_t start, end;       /* first/last bin with H > 1; 0,0 if none */
    uint32_t width;           /* end - start */
    uint32_t visited;         /* bins with H > 0 */
    uint64_t events;          /* sum of H */
    uint64_t min_count;       /* min over all N+1 bins */
    double d_kl;              /* Kullback-Leibler divergence */
    double min_over_mean;     /* min H / mean H over all N+1 bins */
} muca_hist_stats;

/* Options of a full weight-estimation run (muca_delta_multigpu.cu:329-477). */
typedef struct muca_run_opts {
    uint32_t jack;          /* jack index mm (init key 10W + 2*mm) */
    uint32_t starting_M;    /* initial NUPDATES (argv[5]) */
    uint32_t therm;         /* thermalisation attempts per chain per iteration; 0 = N (therm_coeff*N),
                               or 0 for the random-site algorithm (muca_mag.cpp:140) */
    uint32_t rule;          /* muca_update_rule */
    uint32_t hold_until_full; /* 1: no update before width==N (muca_mag.cpp:170-177 intent);
                                 0: update every iteration (what the GPU program does, :466) */
    uint32_t flat_minmean;  /* 0: stop at width==N && D_KL<1e-4 (:447); 1: stop at min/mean >= 0.5 */
    uint32_t max_iter;      /* iteration cap (0 = 1000000) */
    uint32_t init_scheme;   /* muca_init_scheme for the chains; MUCA_INIT_WEIGHT for parity */
    uint32_t reinit_chains; /* 1: initialise chains at the start (the reference does, :340-354) */
    uint32_t nup_schedule;  /* 0: reference ((NUP+1)*1.01 once width==N, :379-382); 1: doubling once
                               width==N; 2: doubling every iteration from the first (cap 2^30);
                               3: as 0, and doubling once every bin also holds >= 5 % of the mean;
                               4: NUP*1.05 every iteration, the first included (muca_mag.cpp:131);
                               5: NUP held until width==N, then NUP*1.05 per iteration (the GPU
                               program's hold, :379-382, with the CPU program's growth, muca_mag.cpp:131) */
    double min_over_mean;   /* threshold for flat_minmean (0 = 0.5) */
    double d_kl_max;        /* threshold of the D_KL test (0 = 1e-4) */
    uint32_t width_start;   /* initial running width (0 = 10, :314); the reference keeps the
                               previous jack's width for jack > 0 */
    uint32_t nup_max;       /* cap of NUPDATES (0: none for schedule 0, 2^30 for the doubling ones) */
    uint32_t graph_iters;   /* 0: one host round trip per iteration, as the reference loop (records carry
                               per-iteration kernel times); K > 0: K iterations per CUDA-graph replay
                               (iterations after the stop do nothing; records carry no kernel times);
                               ignored by muca_weight_run_stream */
} muca_run_opts;

typedef struct muca_iter_record {
    uint32_t k, width_temp, width, nupdates;
    uint64_t total_run;
    double d_kl, min_over_mean, kernel_ms, memcpy_ms;
} muca_iter_record;

typedef struct muca_run_result {
    uint32_t iterations, converged, width_reached_iter;
    uint64_t total_run, nwidth_step;
    double total_kernel_s, total_mem_s, nwidth_time_s, wall_s;
} muca_run_result;

/* Observables of one reweighted production histogram
 * (produce2_multigpu.cu:498-518, plus the Binder cumulant as an extension). */
typedef struct muca_observables {
    double m_abs;   /* <|M|> (not divided by N, as in the reference) */
    double chi;     /* beta (<M^2> - <|M|>^2) / N */
    double u4;      /* 1 - <M^4> / (3 <M^2>^2) */
    double sum, m1, m2, m4;
} muca_observables;

/* ---------------------------------------------------------------------- */
/* Context.  Replaces the per-device set-up of main() in
 * muca_delta_multigpu.cu:93-205 / produce2_multigpu.cu:103-275. */
muca_status muca_create(const muca_params *params, muca_ctx **out);
muca_status muca_destroy(muca_ctx *ctx);
const char *muca_last_error(const muca_ctx *ctx);
muca_status muca_get_info(const muca_ctx *ctx, muca_info *out);
/* reference NUM_WORKERS formula of the device (muca_delta_multigpu.cu:100-106) */
muca_status muca_default_chains(int32_t device, uint32_t *out);
/* Widens the bound of the fast acceptance test (muca_info.log_bracket) to
 * `bracket`, which must lie between the measured bound and 1e30.  (No
 * reference counterpart: the reference always evaluates logf.)  Windows
 * whose decision falls inside the bound are replayed with the exact logf
 * (and, in production, the FP64 difference); 1e30 sends every window there,
 * which checks the exact path on its own.  A bound below the measured one is
 * refused: the fast test could then decide attempts it gets wrong. */
muca_status muca_set_log_bracket(muca_ctx *ctx, double bracket);

/* Failure detection (no reference counterpart: the reference's only check is
 * cudaGetLastError, muca_delta_multigpu.cu:417-421, and its iteration loop has
 * no cap, :374).  Every device-side wait of the warp-specialised sweep gives
 * up after `cycles` SM clock cycles without progress (0 = the default 2^34,
 * about 8 s at 2 GHz; at most 2^40); the launch then ends normally, sets the
 * context's error word, and the next synchronising call returns
 * MUCA_ERR_TIMEOUT (and clears the word, so the context stays usable; the
 * chains' state after such a launch is not valid).  The bound is per wait, so
 * a long launch that keeps making progress never times out. */
muca_status muca_set_wait_limit(muca_ctx *ctx, uint64_t cycles);
/* Test hooks, for tests only (0 in normal use).
 * MUCA_HOOK_SILENT_PRODUCER: the producer warps of the warp-specialised sweep
 * never signal a filled ring slot, so the consumers' bounded waits run out.
 * Nothing faults and every wait stays bounded.
 * MUCA_HOOK_FLUSH_ROWS: the windowed sweep flushes its shared u32 histogram
 * bins into the device histogram before every row it records, the path a
 * launch takes when its bins could otherwise reach 2^32 (results are the
 * same bit for bit). */
#define MUCA_HOOK_SILENT_PRODUCER 1u
#define MUCA_HOOK_FLUSH_ROWS 2u
muca_status muca_set_test_hooks(muca_ctx *ctx, uint32_t hooks);

/* Chains.  Replaces the host lattice init (muca_delta_multigpu.cu:340-354,
 * produce2_multigpu.cu:126-140) and computeEnergies/computeDeltaE/computeM
 * (muca_delta_multigpu.cu:69-83, produce2_multigpu.cu:66-89), on the device. */
muca_status muca_init_chains(muca_ctx *ctx, uint32_t scheme, uint32_t jack);
muca_status muca_set_lattice(muca_ctx *ctx, const int8_t *lat, size_t n);
muca_status muca_get_lattice(muca_ctx *ctx, int8_t *lat, size_t n);
muca_status muca_get_chain_state(muca_ctx *ctx, int32_t *e_j, int32_t *e_delta, int32_t *mag, size_t n);

/* Weights.  Replaces the H2D copy of the FP32 weight (muca_delta_multigpu.cu:384-387)
 * and of the FP64 weight (produce2_multigpu.cu:262). */
muca_status muca_set_weights(muca_ctx *ctx, const double *lnw, size_t n);
muca_status muca_get_weights(muca_ctx *ctx, double *lnw, size_t n);

/* One sweep launch: `therm` attempts per chain, then `nup` attempts per
 * chain with a histogram entry after each.  Replaces one launch of kernel
 * mcs (muca_delta_multigpu.cu:393 / produce2_multigpu.cu:301,311).  The
 * histogram is cleared first (the reference clears it inside the kernel,
 * racily, :746-749).  seed of emulated device d = seed_base + seed_dev_mul*d
 * (the reference passes SEED+1000*l, SEED+1000*GPU+l, SEED+2000*GPU).
 * Random-site algorithm: one call of the CPU program's mcs (muca_mag.cpp:312)
 * for every chain, with WORKER = chain, iter = `iter` and its `seed`
 * argument (the jack index) = seed_base; seed_dev_mul is not used. */
muca_status muca_sweep(muca_ctx *ctx, uint32_t iter, uint32_t seed_base, uint32_t seed_dev_mul,
                       uint64_t therm, uint64_t nup);
/* Same, but accumulate into the histogram instead of clearing it. */
muca_status muca_sweep_accumulate(muca_ctx *ctx, uint32_t iter, uint32_t seed_base, uint32_t seed_dev_mul,
                                  uint64_t therm, uint64_t nup);
muca_status muca_clear_histogram(muca_ctx *ctx);
/* n = N+1 (weight mode) or (N+1)(N+2)/2 (production mode); u64 counts.
 * The reference copies the histogram to the host after every launch
 * (muca_delta_multigpu.cu:404-429, produce2_multigpu.cu:313-316); here it
 * stays on the device and is read only on request.  set_histogram restores
 * a saved histogram (checkpoint/resume, tests). */
muca_status muca_get_histogram(muca_ctx *ctx, uint64_t *h, size_t n);
muca_status muca_set_histogram(muca_ctx *ctx, const uint64_t *h, size_t n);

/* Weight update on the device in FP64.  Replaces the host update
 * muca_delta_multigpu.cu:466-476 (and :833-859 for the recursion); the
 * FP32 shadow used by the next sweep is refreshed.  `stats` (optional)
 * receives the summary of the histogram the update used; with stats == NULL
 * the update is only enqueued on the context's stream (no host wait). */
muca_status muca_histogram_stats(muca_ctx *ctx, muca_hist_stats *stats);
muca_status muca_update_weights(muca_ctx *ctx, uint32_t rule, muca_hist_stats *stats);

/* One iteration of the reference's weight loop with host buffers, as one
 * call with one host synchronisation (muca_delta_multigpu.cu:384-476):
 * lnw_in (N+1 values; NULL keeps the device weights) as muca_set_weights,
 * one sweep as muca_sweep, the update `rule` as muca_update_weights, then
 * the updated weights into lnw_out and the sweep's histogram into hist_out
 * (N+1 each; either may be NULL) and, if stats is not NULL, the histogram
 * summary.  Weight mode only.  The same results as the five separate calls. */
muca_status muca_iterate_host(muca_ctx *ctx, const double *lnw_in, uint32_t iter, uint32_t seed_base,
                              uint32_t seed_dev_mul, uint64_t therm, uint64_t nup, uint32_t rule,
                              double *lnw_out, uint64_t *hist_out, muca_hist_stats *stats);

/* Full weight-estimation run of one jack (muca_delta_multigpu.cu:329-477).
 * recs (optional, capacity cap) receives one record per iteration. */
muca_status muca_weight_run(muca_ctx *ctx, const muca_run_opts *opts, muca_run_result *res,
                            muca_iter_record *recs, size_t cap);
/* Same, calling cb(record, user) on the host after every iteration (the
 * per-iteration log line of :439). */
typedef void (*muca_iter_callback)(const muca_iter_record *rec, void *user);
muca_status muca_weight_run_stream(muca_ctx *ctx, const muca_run_opts *opts, muca_run_result *res,
                                   muca_iter_callback cb, void *user);

/* Production.  Shift lnW (produce2_multigpu.cu:391-400), form
 * boltz_j = exp(-beta*delta*j - lnW_j) (:297) and reweight the current 2D
 * histogram into observables (:498-518), all on the device in FP64.
 * The shift applies to the reweighting copy of the weights only (set by
 * muca_set_weights, shifted cumulatively as the reference shifts its host
 * copy); the sweep keeps the weights as set, as the reference kernel does. */
muca_status muca_weight_shift(muca_ctx *ctx, double beta, double delta);
muca_status muca_get_reweighting_weights(muca_ctx *ctx, double *lnw, size_t n);
muca_status muca_compute_observables(muca_ctx *ctx, double beta, double delta, muca_observables *out);
/* No counterpart in the reference.  The four reweighting sums of
 * muca_compute_observables -- d_sums[0..3] = {sum, m1, m2, m4} -- over a
 * triangular (E_Delta, M) histogram d_hist2d ((N+1)(N+2)/2 u64, N = L*L) and
 * weights d_lnw (N+1 doubles, already shifted as the caller wants), all
 * device buffers owned by the caller; no context.  The call allocates
 * nothing: for callers that must not see a device allocation (a scheduler
 * owning HBM through its own pool and budget; a process that only reweights
 * histograms it holds).  Its scratch is a fixed device array of 304 x 4
 * doubles inside the library (the partials of a fixed 304-block grid; the
 * size does not depend on L), whose address is looked up on the first call
 * per device and cached; make that first call before any stream capture,
 * since it may load the module.  The cached address belongs to the device's
 * current context: after cudaDeviceReset (or anything else that destroys the
 * primary context) it is stale, so do not call this entry point again in
 * that process.  Nothing needs to start at zero.  Two calls in flight at
 * once on the same device share that array and race.  L outside 2..128 is
 * rejected with MUCA_ERR_BAD_ARG: that is the library-wide range of L
 * (muca_create checks the same), not a limit of the scratch.  The caller's current
 * device is the same after the call as before.  The work is enqueued on
 * `stream` (cudaStream_t, NULL = the legacy default stream); d_sums is valid
 * once the stream reaches it.  Errors: muca_last_error(NULL). */
muca_status muca_observables_noalloc(int32_t device, const uint64_t *d_hist2d, const double *d_lnw, uint32_t L,
                                    double beta, double delta, double *d_sums, void *stream);
/* Leave-one-out jackknife (muca_delta_multigpu.cu:620-635) on the device. */
muca_status muca_jackknife(muca_ctx *ctx, const double *x, uint32_t n, double *avg, double *err);

/* Measurement (no reference counterpart): Philox4x32-R blocks per second
 * generated by a full-occupancy kernel in the form the sweeps use, the
 * integer-pipe ceiling against which the sweep kernels are reported. */
muca_status muca_philox_peak(int32_t device, uint32_t rounds, double *blocks_per_s);

/* Measurement (no reference counterpart): the weight-mode windowed sweep
 * taken apart, timed per warp in SM cycles per attempt, in the sweep's
 * geometry at 16384 chains (one block of four warps on one SM, L = 72,
 * lattice, FP32 weights and u32 histogram in shared memory).  part 0: the
 * whole window (draws of the next window, decode, scan, store, histogram);
 * 1: draws and decode alone; 2: scan, store and histogram alone on decoded
 * windows; 3: the bare chain of accept/reject decisions; 4: the draws alone;
 * 5: one dependent FP32 add per attempt slot (its latency); 6: one dependent
 * shared-memory load per attempt slot (its latency).  `windows` (even,
 * 2..2^20) 8-slot windows per lane; the slowest warp is reported.  The
 * caller's current device is the same after the call as before. */
muca_status muca_sweep_floor(int32_t device, uint32_t part, uint32_t windows, double *cycles_per_attempt);

/* ---- Batches of independent weight runs (no counterpart in the reference) ----
 * The reference estimates one (L, T) weight per program run.  A batch runs
 * many such estimations of uneven size together on one GPU: every iteration
 * sweeps all running instances in one persistent kernel and updates each
 * instance's FP64 weights on the device; the iteration loop is captured
 * into a CUDA graph and replayed until every instance has stopped.
 * Instance i is the reference weight loop (muca_delta_multigpu.cu:374-477)
 * for its L and beta with the seeds of emulated device `seed`: initial spins
 * from key {10W, 0xdecafbad}, counter {2*seed, 100, 0xBADCAB1E, 0xBADC0DED};
 * sweep counter word 1 = 100 + 1000*seed.  With beta = 2 its results equal a
 * single context's (muca_params.dev_offset = seed, same L and nchains).
 * Any other beta replaces the reference's -2 dE (T = 0.5, :810) by the
 * FP32 value (float)(-beta*dE). */
typedef struct muca_batch muca_batch;

typedef struct muca_instance {
    uint32_t L;        /* 8..128, a multiple of 8 */
    uint32_t nchains;  /* 1..65536 */
    uint32_t seed;     /* emulated device index of the instance's streams */
    uint32_t reserved;
    double beta;       /* 1/T > 0; 2 is the reference's fixed T = 0.5 */
} muca_instance;

typedef struct muca_batch_shape {
    uint32_t chains_per_block;  /* 32, 64, 128 or 256 */
    uint32_t lattice_in_smem;   /* packed lattice staged in shared memory: 0 no, 1 yes, 2 for the
                                   instances whose block fits (global memory for the rest) */
    uint32_t hist_in_smem;      /* u32 histogram bins in shared memory (else u64 device atomics) */
    uint32_t blocks_per_sm;     /* resident blocks of the persistent grid per SM */
    double ms;                  /* autotuner: one sweep (therm N + nup N) of the whole batch */
} muca_batch_shape;

typedef struct muca_batch_params {
    int32_t device;
    uint32_t rounds;                 /* Philox rounds: 7 (reference) or 10 */
    void *stream;                    /* cudaStream_t; NULL = own stream */
    uint32_t shape_chains_per_block; /* 0 = autotune; else this fixed shape: */
    uint32_t shape_lattice_in_smem;
    uint32_t shape_hist_in_smem;
} muca_batch_params;

typedef struct muca_batch_info {
    uint32_t n_instances, n_items, grid, threads, smem_bytes, n_tried;
    muca_batch_shape shape;     /* in use */
    muca_batch_shape tried[32]; /* the autotuner's table (n_tried entries) */
    uint64_t device_bytes;
    double log_bracket;
} muca_batch_info;

typedef struct muca_batch_run_opts {
    uint32_t starting_M;    /* initial NUPDATES of every instance */
    uint32_t rule;          /* muca_update_rule */
    uint32_t nup_schedule;  /* 0: (NUP+1)*1.01 once width == N (:379-382); 1: doubling once width == N;
                               2: doubling every iteration (cap 2^30); 3: as 0, doubling once every
                               bin also holds >= 5 % of the mean count; 4: NUP*1.05 every iteration,
                               the first included (muca_mag.cpp:131); 5: NUP held until width == N,
                               then NUP*1.05 per iteration */
    uint32_t flat_minmean;  /* 0: stop at width == N && D_KL < d_kl_max; 1: at min/mean >= min_over_mean */
    uint32_t max_iter;      /* per instance (0 = 1000000) */
    uint32_t graph_iters;   /* iterations per captured graph (0 = 16) */
    uint32_t reinit_chains; /* 1: initial spins again before the run */
    uint32_t nup_max;       /* cap of NUPDATES (0: none for schedule 0, 2^30 for the doubling ones) */
    double min_over_mean;   /* 0 = 0.5 */
    double d_kl_max;        /* 0 = 1e-4 */
    uint32_t starting_sweeps; /* nonzero: instance i starts at NUPDATES = starting_sweeps * N_i
                                 (replaces starting_M) */
    uint32_t graded_init;   /* with reinit_chains: 1 = MUCA_INIT_GRADED spins (chains spread over
                               E_Delta), 0 = the reference's initial spins */
} muca_batch_run_opts;

typedef struct muca_batch_result {
    uint32_t iterations, converged, width, reach_iter, nupdates, reserved;
    uint64_t total_run;     /* attempts counted by the reference's acc_NUP: sum of NUPDATES * nchains */
    double d_kl, min_over_mean;  /* of the last iteration */
} muca_batch_result;

/* Creates the batch, chooses the block shape (autotuner unless fixed) and
 * initialises the chains; weights start at zero. */
muca_status muca_batch_create(const muca_batch_params *params, const muca_instance *inst, uint32_t n,
                              muca_batch **out);
muca_status muca_batch_destroy(muca_batch *b);
const char *muca_batch_last_error(const muca_batch *b); /* NULL: errors of muca_batch_create */
muca_status muca_batch_get_info(const muca_batch *b, muca_batch_info *info);
muca_status muca_batch_init_chains(muca_batch *b);
/* Weights of instance i (N+1 values; the warm start of a run) and its results. */
muca_status muca_batch_set_weights(muca_batch *b, uint32_t i, const double *lnw, size_t n);
muca_status muca_batch_get_weights(muca_batch *b, uint32_t i, double *lnw, size_t n);
muca_status muca_batch_get_histogram(muca_batch *b, uint32_t i, uint64_t *hist, size_t n);
/* Runs every instance to its stop criterion or max_iter; res (n entries,
 * may be NULL) gets each instance's outcome, *seconds (may be NULL) the
 * device time.  MUCA_ERR_NOT_CONVERGED if some instance hit max_iter. */
muca_status muca_batch_run(muca_batch *b, const muca_batch_run_opts *opts, muca_batch_result *res,
                           double *seconds);

/* ---- Learned warm start (no counterpart in the reference) ----
 * A multilayer perceptron (L/128, T, Delta, E_Delta/N) -> (lnW - mean lnW)/N,
 * three hidden layers of 128 SiLU units, FP32, trained with Adam on the
 * device by this library's own kernels.  Its prediction replaces the zero or
 * extrapolated initial weight of the reference's `continuing` path
 * (muca_delta_multigpu.cu:223-235); the weight iteration then runs to its
 * usual stop criterion.  Parameters: one flat FP32 array of
 * muca_mlp_param_count() values, per layer the [out][in] matrix then the bias. */
typedef struct muca_mlp muca_mlp;
size_t muca_mlp_param_count(void);
/* seed: initial parameters uniform in +-1/sqrt(fan_in) from splitmix64(seed) */
muca_status muca_mlp_create(int32_t device, uint64_t seed, void *stream, muca_mlp **out);
muca_status muca_mlp_destroy(muca_mlp *m);
const char *muca_mlp_last_error(const muca_mlp *m); /* NULL: errors of muca_mlp_create */
muca_status muca_mlp_get_params(muca_mlp *m, float *params, size_t n);
/* also resets the Adam moments and step count */
muca_status muca_mlp_set_params(muca_mlp *m, const float *params, size_t n);
/* training set: x [n][4] = (L/128, T, Delta, E_Delta/N), t [n] = (lnW - mean)/N */
muca_status muca_mlp_set_data(muca_mlp *m, const float *x, const float *t, uint32_t n);
/* `steps` Adam steps (lr, beta 0.9/0.999, eps 1e-8) on minibatches of `batch`
 * points drawn with Philox(seed, step); losses (steps values, may be NULL)
 * gets each step's mean squared error. */
muca_status muca_mlp_train(muca_mlp *m, uint32_t steps, uint32_t batch, float lr, uint32_t seed, float *losses);
/* gradient of the mean squared error over (x, t) (n points) without a step */
muca_status muca_mlp_grad(muca_mlp *m, const float *x, const float *t, uint32_t n, float *grad, float *loss);
muca_status muca_mlp_predict(muca_mlp *m, const float *x, uint32_t n, float *y);
/* lnW[0..N] for (L, T, Delta): N * (y(i/N) - y(0)), ready for muca_set_weights */
muca_status muca_mlp_log_weights(muca_mlp *m, uint32_t L, double T, double delta, double *lnw, size_t n);

#ifdef __cplusplus
}
#endif
#endif
