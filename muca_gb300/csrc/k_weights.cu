// k_weights.cu -- histogram statistics and weight updates on the device, FP64.
//
// Replaces the host code that runs after every sweep of the reference weight
// program (muca_delta_multigpu.cu:422-476): hist_range (:573-596), the
// Kullback-Leibler divergence against a uniform distribution over visited
// bins (:598-618), the trivial update lnW -= ln H for H > 1 followed by
// lnW -= lnW[0] (:466-476), and weight_recursion (:833-859).  One block
// serves one histogram of N+1 <= 16385 bins.  Element-wise steps use the
// reference's operation order with explicitly rounded FP64 operations, so
// the updated weights equal the host's up to the last-bit differences of the
// device and host log(); the divergence is a tree sum and agrees to ~1e-15.
#include "muca_device.cuh"
#include "muca_internal.h"

#include <cfloat>

namespace muca {

constexpr int kUpdThreads = 1024;

// Reduction over a block of whole warps; lanes beyond the number of warps
// enter the second stage with the operation's identity.
template <typename T, typename Op>
__device__ T block_reduce(T v, Op op, T *sh)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < nw ? sh[lane] : Op::id();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) sh[0] = v;
    }
    __syncthreads();
    const T r = sh[0];
    __syncthreads();
    return r;
}

struct MinI {
    __device__ int operator()(int a, int b) const { return a < b ? a : b; }
    __device__ static int id() { return 0x7FFFFFFF; }
};
struct MaxI {
    __device__ int operator()(int a, int b) const { return a > b ? a : b; }
    __device__ static int id() { return -0x7FFFFFFF - 1; }
};
struct AddU {
    __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const { return a + b; }
    __device__ static unsigned long long id() { return 0ull; }
};
struct MinU {
    __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const { return a < b ? a : b; }
    __device__ static unsigned long long id() { return ~0ull; }
};
struct AddD {
    __device__ double operator()(double a, double b) const { return a + b; }
    __device__ static double id() { return 0.0; }
};

// The prefix of weight_recursion (muca_delta_multigpu.cu:848-858) over the
// pairs i in [start, end):  x_start = lnW[start],
//   x_{i+1} = x_i + dS_i  if pair i is connected (valid[i]),  else lnW[i+1]
// (a pair with an empty bin leaves lnW[i+1] as it was).  The reference runs
// it as one dependent chain of FP64 additions; here the block of (whole
// warps of) threads splits [start, end) into contiguous chunks, each thread
// composes its chunk's maps x -> x + d / x -> c into one, the block scans
// those compositions (warp shuffles, then the warp totals), and every thread
// replays its chunk from its prefix.  Inside a chunk the additions keep the
// reference's order; across chunks they are grouped by the tree, which moves
// the result by a few units in the last place of the partial sums.
// `inc` holds dS_i and `cval` lnW[i+1] of the pairs; out[i] gets x_{i+1}.
// Must be called by every thread of the block.
struct SegMap {
    double t;  // valid: the added sum; not valid: the constant
    int v;     // 1: x -> x + t, 0: x -> t
};
__device__ __forceinline__ SegMap seg_then(SegMap first, SegMap then)
{
    SegMap r;
    r.v = first.v & then.v;
    r.t = then.v ? __dadd_rn(first.t, then.t) : then.t;
    return r;
}

__device__ void block_segmented_prefix(int start, int end, double x0, const double *__restrict__ inc,
                                       const unsigned char *__restrict__ valid,
                                       const double *__restrict__ cval, double *__restrict__ out)
{
    __shared__ double s_t[32];
    __shared__ int s_v[32];
    const int n = end - start;
    if (n <= 0) return;
    const int nt = (int)blockDim.x, tid = (int)threadIdx.x;
    const int chunk = (n + nt - 1) / nt;
    const int lo = start + tid * chunk, hi = min(lo + chunk, end);
    SegMap a{0.0, 1};
    for (int i = lo; i < hi; ++i) {
        const SegMap e{valid[i] ? inc[i] : cval[i], valid[i] ? 1 : 0};
        a = seg_then(a, e);
    }
    // inclusive scan of the thread maps within the warp
    const int lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
    SegMap sc = a;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        SegMap pr;
        pr.t = __shfl_up_sync(0xffffffffu, sc.t, o);
        pr.v = __shfl_up_sync(0xffffffffu, sc.v, o);
        if (lane >= o) sc = seg_then(pr, sc);
    }
    if (lane == 31) { s_t[wid] = sc.t; s_v[wid] = sc.v; }
    __syncthreads();
    if (wid == 0) {
        SegMap w{lane < nw ? s_t[lane] : 0.0, lane < nw ? s_v[lane] : 1};
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            SegMap pr;
            pr.t = __shfl_up_sync(0xffffffffu, w.t, o);
            pr.v = __shfl_up_sync(0xffffffffu, w.v, o);
            if (lane >= o) w = seg_then(pr, w);
        }
        s_t[lane] = w.t;
        s_v[lane] = w.v;
    }
    __syncthreads();
    // exclusive prefix of this thread: the warps before it, then the lanes before it
    SegMap ex{0.0, 1};
    if (wid > 0) ex = SegMap{s_t[wid - 1], s_v[wid - 1]};
    SegMap lp;
    lp.t = __shfl_up_sync(0xffffffffu, sc.t, 1);
    lp.v = __shfl_up_sync(0xffffffffu, sc.v, 1);
    if (lane > 0) ex = seg_then(ex, lp);
    double x = ex.v ? __dadd_rn(x0, ex.t) : ex.t;
    for (int i = lo; i < hi; ++i) {
        x = valid[i] ? __dadd_rn(x, inc[i]) : cval[i];
        out[i] = x;
    }
    __syncthreads();
}

// Statistics of hist[0..N], then (if the update is due) the weight update.
// ctl == nullptr: standalone call, update iff rule >= 0.
// ctl != nullptr: one iteration of a device-driven run (see RunCtl).
// NUPDATES of the next iteration.  sched 0: the reference's (NUP+1)*1.01
// once the width is full (muca_delta_multigpu.cu:379-382); 1: doubling once
// the width is full; 2: doubling every iteration; 3: the reference's growth
// once the width is full and doubling once, in addition, every bin of this
// iteration's histogram holds at least 5 % of the mean count (`covered`);
// 4: NUP * 1.05 every iteration, truncated (the CPU program,
// muca_mag.cpp:131); 5: NUP held until the width is full (as the reference
// GPU program holds it, :379-382), then NUP * 1.05 per iteration (the CPU
// program's growth).  The result is capped at `cap` (0: no cap for sched 0,
// 2^30 otherwise) but never falls below nup.
__host__ __device__ __forceinline__ uint32_t next_nupdates(uint32_t nup, bool full, bool covered, uint32_t sched,
                                                           uint32_t cap)
{
    unsigned long long nx = nup;
    if (sched == 2 || (sched == 1 && full) || (sched == 3 && full && covered)) {
        nx = 2ull * nup;
        if (cap == 0) cap = 1u << 30;
    } else if ((sched == 0 || sched == 3) && full) {
        const unsigned nu = nup + 1u;
        nx = (unsigned)(nu * 1.01);
    } else if (sched == 4 || (sched == 5 && full)) {
        nx = (unsigned long long)((double)nup * 1.05);
        if (cap == 0) cap = 1u << 30;
    }
    if (cap != 0 && nx > cap) nx = cap > nup ? cap : nup;
    return (uint32_t)nx;
}

// The statistics' consumers, one thread: the stats record, and in a
// device-driven run the running width, convergence, record and NUPDATES of
// the next iteration (muca_delta_multigpu.cu:431-447,464-466).  Returns
// whether the weights are to be updated.
__device__ __forceinline__ int bookkeep(int start, int end, unsigned long long vis, unsigned long long ev,
                                        unsigned long long mn, double kl, uint32_t N, int rule,
                                        HistStatsDev *__restrict__ stats, RunCtl *__restrict__ ctl)
{
    const double mean = __ddiv_rn((double)ev, (double)(N + 1));
    const double mom = mean > 0 ? __ddiv_rn((double)mn, mean) : 0.0;
    if (stats) {
        stats->start = start;
        stats->end = end;
        stats->width = (uint32_t)(end - start);
        stats->visited = (uint32_t)vis;
        stats->events = ev;
        stats->min_count = mn;
        stats->d_kl = kl;
        stats->min_over_mean = mom;
    }
    int upd = rule >= 0;
    if (ctl) {
        IterState &st = ctl->st;
        const uint32_t wt = (uint32_t)(end - start);
        st.width_temp = wt;
        if (wt > st.width) st.width = wt;
        if (st.width == N && !st.reach) { st.reach = 1; st.reach_k = st.k; st.nwidth_step = st.total_run; }
        const bool conv = ctl->flat_minmean ? (mom >= ctl->mom_thr) : (st.width == N && kl < ctl->dkl_max);
        const uint32_t ri = ctl->rec_ring ? (ctl->rec_cap ? st.k % ctl->rec_cap : 0u) : st.k;
        if (ri < ctl->rec_cap && ctl->recs) {
            IterRecordDev &r = ctl->recs[ri];
            r.k = st.k; r.width_temp = wt; r.width = st.width; r.nupdates = st.nup;
            r.total_run = st.total_run; r.d_kl = kl; r.min_over_mean = mom;
        }
        upd = !conv && (!ctl->hold || st.width == N);
        if (conv) {
            st.converged = 1;
            st.stop = 1;
        } else {
            st.k += 1;
            if (st.k >= ctl->max_iter) {
                st.stop = 1;
            } else {
                st.nup = next_nupdates(st.nup, st.width == N, mom >= 0.05, ctl->sched, ctl->nup_max);
                st.total_run += (unsigned long long)st.nup * ctl->nchains_total;
            }
        }
    }
    return upd;
}

// Pair i of weight_recursion (muca_delta_multigpu.cu:850-856): for i in
// [start, end) with H_i, H_{i+1} both nonzero,
//   p = H_i H_{i+1} / (H_i + H_{i+1}),  k = p / (p + p_acc[i]),
//   dS_i = (lnW[i+1] - lnW[i]) + k ln(H_i / H_{i+1}),  p_acc[i] += p;
// returns whether the pair is connected (ds[i] written).
__device__ __forceinline__ unsigned char recursion_increment(const unsigned long long *__restrict__ hist,
                                                             const double *__restrict__ lnw,
                                                             double *__restrict__ p_acc, uint32_t i, int start,
                                                             int end, double *__restrict__ ds)
{
    if ((int)i < start || (int)i >= end) return 0;
    const unsigned long long a = hist[i], b = hist[i + 1];
    if ((a == 0) | (b == 0)) return 0;
    const double p = __ddiv_rn((double)(a * b), (double)(a + b));
    const double k = __ddiv_rn(p, __dadd_rn(p, p_acc[i]));
    const double lg = log(__ddiv_rn((double)a, (double)b));
    ds[i] = __dadd_rn(__dadd_rn(-lnw[i], lnw[i + 1]), __dmul_rn(k, lg));
    p_acc[i] = __dadd_rn(p_acc[i], p);
    return 1;
}

// `dyn`: dynamic shared memory of update_smem(N, rule) bytes.
__device__ __forceinline__ void weight_update_body(const unsigned long long *__restrict__ hist, uint32_t N,
                                                   double *__restrict__ lnw, float *__restrict__ w32,
                                                   double *__restrict__ p_acc, int rule,
                                                   HistStatsDev *__restrict__ stats, RunCtl *__restrict__ ctl,
                                                   unsigned char *dyn)
{
    __shared__ int shi[32];
    __shared__ unsigned long long shu[32];
    __shared__ double shd[32];
    __shared__ int do_update;
    const uint32_t tid = threadIdx.x, bs = blockDim.x;
    if (ctl && ctl->st.stop) return;

    // values needed before anything is written (normalisation constant)
    const unsigned long long h0 = hist[0];
    const double lnw0 = lnw[0];

    int lo = (int)N + 1, hi = -1;
    unsigned long long vis = 0, ev = 0, mn = ~0ull;
    for (uint32_t i = tid; i <= N; i += bs) {
        const unsigned long long h = hist[i];
        if (h > 1) { lo = min(lo, (int)i); hi = max(hi, (int)i); }
        if (h > 0) { ++vis; ev += h; }
        mn = h < mn ? h : mn;
    }
    lo = block_reduce(lo, MinI(), shi);
    hi = block_reduce(hi, MaxI(), shi);
    vis = block_reduce(vis, AddU(), shu);
    ev = block_reduce(ev, AddU(), shu);
    mn = block_reduce(mn, MinU(), shu);
    int start = lo, end = hi < 0 ? 0 : hi;
    if (start > end) { start = 0; end = 0; }

    // Kullback-Leibler divergence: sum over H>0 of P ln(P/Q), P = H/events, Q = 1/visited
    const double num_event = (double)ev, Q = __ddiv_rn(1.0, (double)vis);
    double kl = 0.0;
    for (uint32_t i = tid; i <= N; i += bs) {
        const unsigned long long h = hist[i];
        if (h > 0) {
            const double P = __ddiv_rn((double)h, num_event);
            kl = __dadd_rn(kl, __dmul_rn(P, log(__ddiv_rn(P, Q))));
        }
    }
    kl = block_reduce(kl, AddD(), shd);
    if (tid == 0) do_update = bookkeep(start, end, vis, ev, mn, kl, N, rule, stats, ctl);
    __syncthreads();
    if (!do_update) return;

    if (rule == 0 || rule == 1) {
        // tmp = lnW[0] after the ln H subtraction (:469), computed from the
        // values read before any write
        const unsigned long long thr = rule == 0 ? 1ull : 0ull;
        const double tmp = h0 > thr ? __dsub_rn(lnw0, log((double)h0)) : lnw0;
        for (uint32_t i = tid; i <= N; i += bs) {
            const unsigned long long h = hist[i];
            double v = lnw[i];
            if (h > thr) v = __dsub_rn(v, log((double)h));
            if (rule == 0 || h > 0) v = __dsub_rn(v, tmp);
            lnw[i] = v;
            w32[i] = (float)v;
        }
        return;
    }

    // rule 2: weight_recursion (:848-858) then lnW -= lnW[0].
    // (a) the increments dS_i of all connected pairs, in parallel;
    double *ds = reinterpret_cast<double *>(dyn);
    unsigned char *valid = dyn + sizeof(double) * (size_t)N;
    for (uint32_t i = tid; i < N; i += bs) valid[i] = recursion_increment(hist, lnw, p_acc, i, start, end, ds);
    __syncthreads();
    // (b) the prefix lnW[i+1] = lnW[i] + dS_i, in place over ds (a pair
    //     with an empty bin leaves lnW[i+1] at its old value);
    block_segmented_prefix(start, end, lnw[start], ds, valid, lnw + 1, ds);
    // (c) write back and normalise by lnW[0] (bin 0 is never rewritten)
    for (uint32_t i = tid; i <= N; i += bs) {
        double v = ((int)i > start && (int)i <= end) ? ds[i - 1] : lnw[i];
        v = __dsub_rn(v, lnw0);
        lnw[i] = v;
        w32[i] = (float)v;
    }
}

__global__ void __launch_bounds__(kUpdThreads) k_weight_update(const unsigned long long *__restrict__ hist, uint32_t N,
                                                                double *__restrict__ lnw, float *__restrict__ w32,
                                                                double *__restrict__ p_acc, int rule,
                                                                HistStatsDev *__restrict__ stats,
                                                                RunCtl *__restrict__ ctl)
{
    extern __shared__ __align__(16) unsigned char dyn[];
    weight_update_body(hist, N, lnw, w32, p_acc, rule, stats, ctl, dyn);
}

// ---- the same statistics and update over kUpdBlocks blocks ---------------
// The divergence terms and the ln H of the update are FP64 per bin, and FP64
// issues slowly on this GPU: one block leaves all of them to one SM (ncu:
// 67 % of that SM's FP64 pipe, 28 us at L=72).  Here pass 1 forms the integer
// statistics per block; pass 2 the divergence terms per block, after every
// block has summed the partial event and visited counts in block order; the
// last block of pass 2 sums all partials in block order, keeps the books as
// the one-block update does (bookkeep) and decides the update; pass 3
// applies it.  Integer statistics and the updated weights equal the one-block
// update's; the divergence sum runs in another order.
constexpr int kUpdMultiThreads = 256;

__global__ void __launch_bounds__(kUpdMultiThreads) k_upd_stats(const unsigned long long *__restrict__ hist,
                                                                uint32_t N, const RunCtl *__restrict__ ctl,
                                                                UpdScratch *__restrict__ sc)
{
    __shared__ int shi[32];
    __shared__ unsigned long long shu[32];
    if (ctl && ctl->st.stop) return;
    int lo = (int)N + 1, hi = -1;
    unsigned long long vis = 0, ev = 0, mn = ~0ull;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= N; i += gridDim.x * blockDim.x) {
        const unsigned long long h = hist[i];
        if (h > 1) { lo = min(lo, (int)i); hi = max(hi, (int)i); }
        if (h > 0) { ++vis; ev += h; }
        mn = h < mn ? h : mn;
    }
    lo = block_reduce(lo, MinI(), shi);
    hi = block_reduce(hi, MaxI(), shi);
    vis = block_reduce(vis, AddU(), shu);
    ev = block_reduce(ev, AddU(), shu);
    mn = block_reduce(mn, MinU(), shu);
    if (threadIdx.x == 0) {
        UpdPart &p = sc->part[blockIdx.x];
        p.lo = lo; p.hi = hi; p.vis = vis; p.ev = ev; p.mn = mn;
    }
}

__global__ void __launch_bounds__(kUpdMultiThreads) k_upd_kl(const unsigned long long *__restrict__ hist, uint32_t N,
                                                             const double *__restrict__ lnw, int rule,
                                                             HistStatsDev *__restrict__ stats,
                                                             RunCtl *__restrict__ ctl, UpdScratch *__restrict__ sc)
{
    __shared__ double shd[32];
    __shared__ unsigned long long s_ev, s_vis;
    __shared__ int s_last;
    if (ctl && ctl->st.stop) {
        // an iteration after the stop: no update either
        if (blockIdx.x == 0 && threadIdx.x == 0) sc->upd = 0;
        return;
    }
    if (threadIdx.x < 32) {
        // the partial counts, two per lane, then a warp sum (fixed order)
        unsigned long long e = 0, v = 0;
        for (uint32_t b = threadIdx.x; b < gridDim.x; b += 32) { e += sc->part[b].ev; v += sc->part[b].vis; }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            e += __shfl_xor_sync(0xffffffffu, e, o);
            v += __shfl_xor_sync(0xffffffffu, v, o);
        }
        if (threadIdx.x == 0) {
            s_ev = e;
            s_vis = v;
        }
    }
    __syncthreads();
    // sum over H>0 of P ln(P/Q), P = H/events, Q = 1/visited (as the one-block update)
    const double num_event = (double)s_ev, Q = __ddiv_rn(1.0, (double)s_vis);
    double kl = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= N; i += gridDim.x * blockDim.x) {
        const unsigned long long h = hist[i];
        if (h > 0) {
            const double P = __ddiv_rn((double)h, num_event);
            kl = __dadd_rn(kl, __dmul_rn(P, log(__ddiv_rn(P, Q))));
        }
    }
    kl = block_reduce(kl, AddD(), shd);
    if (threadIdx.x == 0) {
        sc->part[blockIdx.x].kl = kl;
        __threadfence();
        s_last = atomicAdd(&sc->done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last || threadIdx.x >= 32) return;
    __threadfence();
    // all partials, two per lane, then warp reductions (fixed order)
    int lo = (int)N + 1, hi = -1;
    unsigned long long vis = 0, ev = 0, mn = ~0ull;
    double klt = 0.0;
    for (uint32_t b = threadIdx.x; b < gridDim.x; b += 32) {
        const UpdPart &p = sc->part[b];
        lo = min(lo, p.lo);
        hi = max(hi, p.hi);
        vis += p.vis;
        ev += p.ev;
        mn = p.mn < mn ? p.mn : mn;
        klt = __dadd_rn(klt, __ldcg(&p.kl));  // written by other blocks of this launch
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        vis += __shfl_xor_sync(0xffffffffu, vis, o);
        ev += __shfl_xor_sync(0xffffffffu, ev, o);
        const unsigned long long m2 = __shfl_xor_sync(0xffffffffu, mn, o);
        mn = m2 < mn ? m2 : mn;
        klt = __dadd_rn(klt, __shfl_xor_sync(0xffffffffu, klt, o));
    }
    if (threadIdx.x != 0) return;
    int start = lo, end = hi < 0 ? 0 : hi;
    if (start > end) { start = 0; end = 0; }
    sc->upd = bookkeep(start, end, vis, ev, mn, klt, N, rule, stats, ctl);
    sc->start = start;
    sc->end = end;
    // lnW[0] after its ln H subtraction (:469), from the weights before any write
    const unsigned long long h0 = hist[0], thr = rule == 0 ? 1ull : 0ull;
    sc->tmp = h0 > thr ? __dsub_rn(lnw[0], log((double)h0)) : lnw[0];
    sc->done = 0;
}

__global__ void __launch_bounds__(kUpdMultiThreads) k_upd_apply(const unsigned long long *__restrict__ hist,
                                                                uint32_t N, double *__restrict__ lnw,
                                                                float *__restrict__ w32, int rule,
                                                                const UpdScratch *__restrict__ sc)
{
    if (!sc->upd) return;
    const unsigned long long thr = rule == 0 ? 1ull : 0ull;
    const double tmp = sc->tmp;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= N; i += gridDim.x * blockDim.x) {
        const unsigned long long h = hist[i];
        double v = lnw[i];
        if (h > thr) v = __dsub_rn(v, log((double)h));
        if (rule == 0 || h > 0) v = __dsub_rn(v, tmp);
        lnw[i] = v;
        w32[i] = (float)v;
    }
}

// Rule 2 over kUpdBlocks blocks: the increments of every connected pair
// (FP64 divisions and a logarithm each) ...
__global__ void __launch_bounds__(kUpdMultiThreads) k_upd_rec_inc(const unsigned long long *__restrict__ hist,
                                                                  uint32_t N, const double *__restrict__ lnw,
                                                                  double *__restrict__ p_acc,
                                                                  const UpdScratch *__restrict__ sc, RecScratch rs)
{
    if (!sc->upd) return;
    const int start = sc->start, end = sc->end;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        rs.valid[i] = recursion_increment(hist, lnw, p_acc, i, start, end, rs.ds);
}

// ... then the prefix as one block's segmented scan, the write-back and the
// normalisation by lnW[0] (bin 0 is never rewritten by the recursion).
__global__ void __launch_bounds__(kUpdThreads) k_upd_rec_scan(uint32_t N, double *__restrict__ lnw,
                                                               float *__restrict__ w32,
                                                               const UpdScratch *__restrict__ sc, RecScratch rs)
{
    if (!sc->upd) return;
    const int start = sc->start, end = sc->end;
    const double lnw0 = lnw[0];
    block_segmented_prefix(start, end, lnw[start], rs.ds, rs.valid, lnw + 1, rs.ds);
    for (uint32_t i = threadIdx.x; i <= N; i += blockDim.x) {
        double v = ((int)i > start && (int)i <= end) ? rs.ds[i - 1] : lnw[i];
        v = __dsub_rn(v, lnw0);
        lnw[i] = v;
        w32[i] = (float)v;
    }
}

static cudaError_t launch_update_multi(const unsigned long long *hist, uint32_t N, double *lnw, float *w32,
                                       double *p_acc, int rule, HistStatsDev *stats, RunCtl *ctl, UpdScratch *sc,
                                       const RecScratch *rs, cudaStream_t s)
{
    k_upd_stats<<<kUpdBlocks, kUpdMultiThreads, 0, s>>>(hist, N, ctl, sc);
    k_upd_kl<<<kUpdBlocks, kUpdMultiThreads, 0, s>>>(hist, N, lnw, rule, stats, ctl, sc);
    if (rule == 2) {
        k_upd_rec_inc<<<kUpdBlocks, kUpdMultiThreads, 0, s>>>(hist, N, lnw, p_acc, sc, *rs);
        k_upd_rec_scan<<<1, kUpdThreads, 0, s>>>(N, lnw, w32, sc, *rs);
    } else if (rule >= 0) {
        k_upd_apply<<<kUpdBlocks, kUpdMultiThreads, 0, s>>>(hist, N, lnw, w32, rule, sc);
    }
    return cudaGetLastError();
}

// One iteration's tail for every instance of a batch (block i = instance i),
// then the count of instances that are still running.
__global__ void __launch_bounds__(kUpdThreads) k_batch_update(const BatchInst *__restrict__ insts,
                                                               uint32_t *__restrict__ running)
{
    extern __shared__ __align__(16) unsigned char dyn[];
    const BatchInst &I = insts[blockIdx.x];
    weight_update_body(I.a.hist, I.a.N, I.lnw, I.w32, I.p_acc, (int)I.rule, nullptr, I.ctl, dyn);
    if (threadIdx.x == 0 && !I.ctl->st.stop) atomicAdd(running, 1u);
}

__global__ void k_run_clear(unsigned long long *hist, uint32_t n, const RunCtl *ctl)
{
    if (ctl->st.stop) return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) hist[i] = 0ull;
}

__global__ void k_to_f32(const double *lnw, float *w32, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) w32[i] = (float)lnw[i];
}

static size_t update_smem(uint32_t N, int rule) { return rule == 2 ? (size_t)N * (sizeof(double) + 1) : 0; }

static cudaError_t prep_update(uint32_t N, int rule)
{
    const size_t dyn = update_smem(N, rule);
    if (dyn > 48 * 1024)
        return cudaFuncSetAttribute(k_weight_update, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    return cudaSuccess;
}

cudaError_t launch_weight_update(const unsigned long long *hist, uint32_t N, double *lnw, float *w32, double *p_acc,
                                 int rule, HistStatsDev *stats, cudaStream_t s, UpdScratch *sc, const RecScratch *rs)
{
    if (sc && (rule != 2 || rs)) return launch_update_multi(hist, N, lnw, w32, p_acc, rule, stats, nullptr, sc, rs, s);
    cudaError_t e = prep_update(N, rule);
    if (e != cudaSuccess) return e;
    k_weight_update<<<1, kUpdThreads, update_smem(N, rule), s>>>(hist, N, lnw, w32, p_acc, rule, stats, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_run_update(const unsigned long long *hist, double *lnw, float *w32, double *p_acc, RunCtl *ctl,
                              cudaStream_t s, uint32_t N, int rule, UpdScratch *sc, const RecScratch *rs)
{
    if (sc && (rule != 2 || rs)) return launch_update_multi(hist, N, lnw, w32, p_acc, rule, nullptr, ctl, sc, rs, s);
    cudaError_t e = prep_update(N, rule);
    if (e != cudaSuccess) return e;
    k_weight_update<<<1, kUpdThreads, update_smem(N, rule), s>>>(hist, N, lnw, w32, p_acc, rule, nullptr, ctl);
    return cudaGetLastError();
}

cudaError_t prepare_batch_update(uint32_t max_N, int any_recursion)
{
    const size_t dyn = any_recursion ? update_smem(max_N, 2) : 0;
    if (dyn > 48 * 1024)
        return cudaFuncSetAttribute(k_batch_update, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    return cudaSuccess;
}

cudaError_t launch_batch_update(const BatchInst *insts, uint32_t n_inst, uint32_t max_N, int any_recursion,
                                uint32_t *running, cudaStream_t s)
{
    const size_t dyn = any_recursion ? update_smem(max_N, 2) : 0;
    k_batch_update<<<n_inst, kUpdThreads, dyn, s>>>(insts, running);
    return cudaGetLastError();
}

cudaError_t launch_run_clear(unsigned long long *hist, uint32_t n, const RunCtl *ctl, cudaStream_t s)
{
    k_run_clear<<<(n + 255) / 256 < 152 ? (n + 255) / 256 : 152, 256, 0, s>>>(hist, n, ctl);
    return cudaGetLastError();
}

cudaError_t launch_weights_to_f32(const double *lnw, float *w32, uint32_t n, cudaStream_t s)
{
    k_to_f32<<<(n + 255) / 256, 256, 0, s>>>(lnw, w32, n);
    return cudaGetLastError();
}

}  // namespace muca
