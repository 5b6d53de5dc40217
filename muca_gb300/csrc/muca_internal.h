// muca_internal.h -- launch interfaces between the C ABI (muca_api.cu) and the
// kernel translation units.  Not part of the public ABI.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace muca {

// One sweep launch.  The lattice is packed (see muca_device.cuh); `w` is
// float[N+1] (weight mode) or double[N+1] (production mode); `hist` is
// u64[N+1] or u64[(N+1)(N+2)/2].  Chain c belongs to emulated device
// c / chains_per_dev and uses WORKER = c % chains_per_dev; its Philox keys
// are k1 = {k1_mul*W + k1_add, k1_hi}, k3 = {k3_mul*W + k3_add, k3_hi}, its
// counter {c0, seed_base + seed_dev_mul*dev, iter, 0xBADC0DED}.
struct SweepArgs {
    uint32_t *lat;
    int32_t *ej, *edel, *mag;
    const void *w;
    unsigned long long *hist;
    const uint32_t *index;  // sweep order (generic kernel only), N entries
    const uint32_t *naver;  // neighbours (generic kernel only), 4N entries
    uint32_t L, N, WPR, nchains, chains_per_dev;
    uint32_t seed_base, seed_dev_mul, iter;
    unsigned long long therm, nup;
    uint32_t k1_mul, k1_add, k1_hi, k3_mul, k3_add, k3_hi;
    // bound on |__logf(u) - logf(u)| over all u01fixedpt<float> values
    // (measure_logf_bracket) times a safety factor; 0 disables the fast test
    double log_eps;
    // optional device-resident (iter, nup, skip) for graph-captured loops;
    // when non-null they override iter/nup and a nonzero skip makes the
    // launch a no-op.
    const uint32_t *dyn;
    // error word: bit 0 is set when a bounded wait inside a kernel gave up
    unsigned int *err;
    // bound of every device-side wait (warp-specialised kernel), in SM clock
    // cycles without progress; 0 = kWaitCyclesDefault
    long long wait_cycles;
    // test hooks (kHook*); 0 in normal operation
    uint32_t hooks;
};
// ~8 s at 2 GHz without progress: a healthy wait completes in microseconds
constexpr long long kWaitCyclesDefault = 1ll << 34;
// kHookSilentProducer: the producer warps of the warp-specialised sweep never
// signal a filled ring slot, so the consumers' bounded waits run out and the
// launch ends with the error word set (a test of the timeout path; it faults
// nothing and every wait stays bounded)
constexpr uint32_t kHookSilentProducer = 1u;
// kHookFlushRows: the windowed sweep flushes its shared u32 bins before every
// recorded row, as a launch that could fill a bin does
constexpr uint32_t kHookFlushRows = 2u;

enum SweepMode { kModeWeight = 0, kModeProduce = 1 };

enum SweepKernel { kKernelGeneric = 0, kKernelWindowed = 1, kKernelSpecialized = 2 };

struct SweepPlan {
    int mode;
    int rounds;
    int kernel;      // SweepKernel
    bool fast;       // windowed kernels usable (L % 8 == 0)
    bool lat_smem;   // lattice resident in shared memory
    bool row_ring;   // lattice in global memory behind a four-row ring per lane (windowed kernel)
    uint32_t cpb;    // chains per block (lane stride of the packed lattice)
    uint32_t threads;  // threads per block
    uint32_t blocks;
    size_t smem;     // dynamic shared memory bytes
};
// Warp-specialised sweep: ring slots per warp pair (the producer runs at most
// this many decoded windows ahead), and u32 words per slot and lane.
constexpr uint32_t kRingDepth = 2;
constexpr uint32_t kSlotWords = 30;

// Chooses placement and block shape for (mode, L, nchains) on a device with
// `smem_optin` bytes of opt-in shared memory per block and `sms` SMs.
// kernel: -1 = choose (windowed when L % 8 == 0, else generic), else a SweepKernel.
SweepPlan plan_sweep(int mode, int rounds, uint32_t L, uint32_t nchains, size_t smem_optin, int sms, int kernel = -1);
// Worst case of |__logf(u) - logf(u)| over u = (2k+1) 2^-24, k < 2^23 (exhaustive, on the device).
cudaError_t measure_logf_bracket(float *max_abs_err, cudaStream_t s);
// The bound of the fast acceptance test for `device` (current): twice the
// measured worst case, measured once per device and cached; 1e30 (every
// decision on the exact logf) if the measurement is implausible.
cudaError_t device_log_eps(int device, cudaStream_t s, double *eps);
cudaError_t launch_sweep(const SweepPlan &p, const SweepArgs &a, cudaStream_t s);

// Random-site sweep of the reference's CPU weight program (k_sweep_random.cu,
// muca_mag.cpp:312-393): chain c is WORKER worker0 + c, `seed` the jack
// index; FP64 weights w[N+1]; logf_tab (2^23 floats, entry k = log of
// (2k+1) 2^-24) gives the acceptance logarithm, NULL = CUDA's logf.
struct RandomArgs {
    uint32_t *lat;
    int32_t *ej, *edel;
    const double *w;
    unsigned long long *hist;
    uint32_t L, N, WPR, nchains, worker0, seed, iter;
    unsigned long long therm, nup;
    const float *logf_tab;
    const uint32_t *dyn;  // as SweepArgs::dyn
    // bound on |__logf(u) - log(u)| over every u01fixedpt<float> value, log
    // being logf_tab's values (when given) or CUDA's logf, with a safety factor
    double log_eps;
    // ceil(2^32 / L): row = high 32 bits of idx * inv_L for idx < N <= 2^14
    uint32_t inv_L;
};
// Worst case of |__logf(u) - tab[k]| over u = (2k+1) 2^-24, k < 2^23 (exhaustive, on the device).
cudaError_t measure_table_bracket(const float *tab, float *max_abs_err, cudaStream_t s);
size_t random_sweep_smem(uint32_t L, uint32_t cpb, bool lat_smem);
// Block shape of the random-site sweep for (L, nchains) on a device with
// `smem_optin` bytes of opt-in shared memory per block and `sms` SMs.
SweepPlan plan_random(uint32_t L, uint32_t nchains, size_t smem_optin, int sms);
cudaError_t launch_sweep_random(const RandomArgs &a, uint32_t cpb, uint32_t blocks, int rounds, size_t smem_optin,
                                cudaStream_t s);

// Lattice helpers (k_lattice.cu).
// key = {key0_mul*W + key0_jack_mul*jack + key0_add, key1 + key1_jack_mul*jack}
struct InitArgs {
    uint32_t key0_mul, key0_jack_mul, key0_add, key1, key1_jack_mul;
    uint32_t ctr0[4], ctr0_dev_mul[4];
    uint32_t ctr_word;  // counter word incremented before every 4 sites
    uint32_t rounds;
    uint32_t chain_in_ctr;  // 1: ctr[0] = chain_offset + chain and ctr[1] = group (chain-counter scheme)
    uint32_t chain_offset;
    uint32_t ordered;       // 1: every spin +1
    uint32_t graded;        // 1: graded_spin of the same Philox words instead of init_spin
};
cudaError_t launch_init(uint32_t *lat, uint32_t L, uint32_t WPR, uint32_t cpb, uint32_t nchains,
                        uint32_t chains_per_dev, uint32_t jack, const InitArgs &ia, cudaStream_t s);
cudaError_t launch_pack(uint32_t *lat, const int8_t *src, uint32_t L, uint32_t WPR, uint32_t cpb,
                        uint32_t nchains, cudaStream_t s);
cudaError_t launch_unpack(const uint32_t *lat, int8_t *dst, uint32_t L, uint32_t WPR, uint32_t cpb,
                          uint32_t nchains, cudaStream_t s);
cudaError_t launch_energies(const uint32_t *lat, int32_t *ej, int32_t *edel, int32_t *mag, uint32_t L,
                            uint32_t WPR, uint32_t cpb, uint32_t nchains, cudaStream_t s);
// Checks that every value of an int8 lattice is in {-1,0,1}; *bad gets the count of others.
cudaError_t launch_validate(const int8_t *src, size_t n, unsigned long long *bad, cudaStream_t s);

// Weight math (k_weights.cu), FP64, one block per instance.
struct HistStatsDev {
    int32_t start, end;
    uint32_t width, visited;
    unsigned long long events, min_count;
    double d_kl, min_over_mean;
};
// Scratch of the multi-block weight update of one context: per-block
// partial statistics, the count of finished blocks, and the decision the
// last block takes for the update pass.
constexpr uint32_t kUpdBlocks = 64;
struct UpdPart {
    int lo, hi;
    unsigned long long vis, ev, mn;
    double kl;
};
struct UpdScratch {
    UpdPart part[kUpdBlocks];
    unsigned int done;
    int upd;
    double tmp;
    int start, end;  // the histogram's range (bins with H > 1), for the recursion
};
// Global scratch of the multi-block recursion: dS_i (N doubles) and the
// connected-pair flags (N bytes).
struct RecScratch {
    double *ds;
    unsigned char *valid;
};
// stats of hist[0..N]; if rule >= 0 also updates lnw (FP64) / w32 (FP32 shadow)
// (rule: 0 trivial, 1 trivial-cpu, 2 recursion with p_acc).  With `sc`
// (zero-initialised once) rules -1, 0 and 1 spread their FP64 work over
// kUpdBlocks blocks, and so does rule 2 when `rs` is given too (its prefix
// then runs as one block's segmented scan); otherwise one block does all.
cudaError_t launch_weight_update(const unsigned long long *hist, uint32_t N, double *lnw, float *w32,
                                 double *p_acc, int rule, HistStatsDev *stats, cudaStream_t s,
                                 UpdScratch *sc = nullptr, const RecScratch *rs = nullptr);

// Device-resident state of a weight-estimation run (the loop of
// muca_delta_multigpu.cu:374-477).  The first three words are what the
// sweep kernel reads through SweepArgs::dyn: iteration index, NUPDATES of
// this iteration, stop flag.
struct IterState {
    uint32_t k, nup, stop, width;
    uint32_t reach, reach_k, converged, width_temp;
    unsigned long long total_run, nwidth_step;
};
struct IterRecordDev {
    uint32_t k, width_temp, width, nupdates;
    unsigned long long total_run;
    double d_kl, min_over_mean;
};
struct RunCtl {
    IterState st;
    uint32_t N, nchains_total, rule, hold, flat_minmean, max_iter, sched, rec_cap;
    uint32_t rec_ring;  // 1: records go to recs[k % rec_cap] (streaming), else recs[k] for k < rec_cap
    uint32_t nup_max;   // cap of NUPDATES (0: none for schedule 0, 2^30 for the doubling ones)
    double mom_thr, dkl_max;
    IterRecordDev *recs;
};
// One instance of a batch of weight runs: its sweep arguments (a.dyn points
// at ctl->st, a.w at w32), its run state and its FP64 weights.  btab[dE + 8]
// = (float)(-beta * dE) for dE = -8..8, the Metropolis term of any beta.
struct BatchInst {
    SweepArgs a;
    RunCtl *ctl;
    double *lnw, *p_acc;
    float *w32;
    float btab[17];
    uint32_t rule;
};
// A unit of sweep work: chain block `blk` of instance `inst`.
struct BatchItem {
    uint32_t inst, blk;
};
// Clears the histograms of the running instances and resets the work counter.
cudaError_t launch_batch_prep(const BatchInst *insts, uint32_t n_inst, uint32_t *next_item, uint32_t *running,
                              cudaStream_t s);
// Lattice placement of a batch sweep: in global memory, in shared memory,
// or per instance in shared memory where it fits in the block's `smem`
// bytes (global memory for the rest).
enum BatchLattice : uint32_t { kLatGlobal = 0, kLatShared = 1, kLatWhereFits = 2 };
// Persistent sweep over `items` (fetched through *next_item) with chain
// blocks of cpb chains; lat (BatchLattice) / hist_smem select the
// shared-memory placement.  grid blocks of roundup32(cpb) threads and
// `smem` bytes.
cudaError_t launch_batch_sweep(const BatchInst *insts, const BatchItem *items, uint32_t n_items, uint32_t *next_item,
                               uint32_t cpb, int rounds, uint32_t lat, bool hist_smem, uint32_t grid, size_t smem,
                               cudaStream_t s);
// Dynamic shared memory of one batch sweep block for an instance of size L,
// with its lattice, or without it (then optionally with its four-row ring).
size_t batch_sweep_smem(uint32_t L, uint32_t cpb, bool lat_smem, bool hist_smem, bool row_ring = false);
// Blocks of the batch sweep that fit on one SM with `smem` bytes each; also
// sets the kernel's shared-memory limit to `smem` (call before any capture).
// The launch with that shape needs no further attribute call.
cudaError_t batch_sweep_occupancy(uint32_t cpb, int rounds, uint32_t lat, bool hist_smem, size_t smem, int *blocks);
// Sets the update kernel's shared-memory limit (call before any capture).
cudaError_t prepare_batch_update(uint32_t max_N, int any_recursion);
// The update step of every instance; *running += instances not stopped.
cudaError_t launch_batch_update(const BatchInst *insts, uint32_t n_inst, uint32_t max_N, int any_recursion,
                                uint32_t *running, cudaStream_t s);

// One iteration's tail: statistics, width/convergence bookkeeping, weight
// update, schedule of the next NUPDATES; a no-op once st.stop is set.
cudaError_t launch_run_update(const unsigned long long *hist, double *lnw, float *w32, double *p_acc,
                              RunCtl *ctl, cudaStream_t s, uint32_t N, int rule, UpdScratch *sc = nullptr,
                              const RecScratch *rs = nullptr);
// Clears the weight histogram unless the run has stopped.
cudaError_t launch_run_clear(unsigned long long *hist, uint32_t n, const RunCtl *ctl, cudaStream_t s);
cudaError_t launch_weights_to_f32(const double *lnw, float *w32, uint32_t n, cudaStream_t s);

// Production reweighting (k_observables.cu).
cudaError_t launch_weight_shift(double *lnw, uint32_t N, double beta, double delta, cudaStream_t s);
// Sums {sum, M1, M2, M4} over the triangular histogram with boltz_i =
// exp(-beta*delta*i - lnw_i) into out[4] (device), using `partials`
// (device, at least observables_partials(N) doubles) as scratch.
size_t observables_partials(uint32_t N);
cudaError_t launch_observables(const unsigned long long *hist2d, const double *lnw, uint32_t N, double beta,
                               double delta, double *partials, double *out, cudaStream_t s);
cudaError_t launch_jackknife(const double *x, uint32_t n, double *out2, cudaStream_t s);
// The same sums with the partials in a file-scope device array of
// observables_static_partials() doubles (no allocation); `device` must be the
// current device.  Calls in flight at once on one device race on that array.
size_t observables_static_partials();
cudaError_t launch_observables_static(int device, const unsigned long long *hist2d, const double *lnw, uint32_t N,
                                      double beta, double delta, double *out, cudaStream_t s);

// Warm-start MLP (k_mlp.cu): 4 -> 128 -> 128 -> 128 -> 1, SiLU, FP32.
size_t mlp_param_count();
cudaError_t mlp_prepare();  // shared-memory limits (call before any capture)
// scratch floats of a minibatch of B points: Xb [B][4] at 0, Tb [B] at 4B,
// Y [B] at 5B, then (aligned) Z, dZ and partials
size_t mlp_scratch_floats(uint32_t B);
// Y[0..B) = net(Xb) (Z: pre-activations [3][B][128] or NULL)
cudaError_t launch_mlp_forward(const float *P, const float *Xb, uint32_t B, float *Z, float *Y, cudaStream_t s);
// Gradient of the mean squared error on a minibatch (drawn from (X, T, n)
// when gather, else already in scratch) into G; with m and v also one Adam
// step; the loss goes to losses[*step - *base] (or losses[0] without step).
cudaError_t launch_mlp_step(float *P, float *G, float *m, float *v, const float *X, const float *T, uint32_t n,
                            uint32_t B, uint32_t *step, const uint32_t *base, uint32_t seed, bool gather, float lr,
                            float *scratch, float *losses, uint32_t losses_cap, cudaStream_t s);

// Philox throughput microbenchmark (k_bench.cu): grid blocks of 256 threads,
// each generating blocks_per_thread Philox4x32-R blocks.
cudaError_t launch_philox_peak(int rounds, uint32_t grid, uint32_t blocks_per_thread, uint32_t *out, cudaStream_t s);
// the weight-mode windowed sweep taken apart (part 0..3), cycles per warp of `windows` 8-site windows
cudaError_t launch_sweep_floor(int part, uint32_t windows, unsigned long long *cycles, uint32_t *sink,
                               unsigned long long *hist_dummy, cudaStream_t s);

}  // namespace muca
