// k_sweep.cu -- Metropolis sweep kernels of the multicanonical hot path.
//
// One chain per thread, as in the reference kernels mcs
// (muca_delta_multigpu.cu:737-829, weight estimation, FP32 weights, 1D
// histogram of E_Delta) and mcs (produce2_multigpu.cu:401-496, production,
// FP64 weights, M tracked, 2D (E_Delta, M) histogram).  Every attempt
// reproduces the reference's arithmetic: same Philox4x32 keys and counters,
// same sweep order (even linear sites, then odd ones: :173), same proposal
// (s -> s +/- 1 with the cyclic wrap of :802), same
//   diff = (float)(-2 dE) + w[E + dDel] - w[E]        (:810)
// evaluated without contraction, and the same test diff >= 0 || logf(u) < diff.
//
// GB300 layout (fast kernel, L % 8 == 0):
//   * the lattice lives in shared memory, 2 bits per spin, rows padded to
//     16-site words, [word][lane] so a warp's 32 chains hit 32 banks;
//   * the weights (FP32 or FP64) and, in weight mode, a u32 histogram live in
//     shared memory; the histogram is flushed to the u64 device histogram
//     once per launch (the reference does one global atomic per attempt);
//   * the sweep is processed in windows of the 8 (or 4) same-parity sites of
//     one word of one row.  Sites of a window are never neighbours of each
//     other (their neighbours are the other parity or the rows above/below),
//     so the whole window's proposals and energy changes are formed from four
//     word loads with nibble-parallel (SWAR) arithmetic; only the
//     accept/reject scan over E_Delta is sequential.  The window's new spins
//     are merged into one word store;
//   * the acceptance test uses the hardware __logf(u) and falls back to the
//     exact logf(u) (replaying the window) whenever __logf(u) lies within the
//     measured worst-case difference of the two functions from diff in any
//     lane, so every decision equals the reference's logf decision;
//   * the Philox blocks of the next window are generated while the current
//     window's sequential scan runs (a two-group queue), so the integer work
//     fills the latency of the scan.
// The generic kernel (any L) follows the reference step by step on the same
// packed layout and is used for L % 8 != 0.
#include "muca_device.cuh"
#include "muca_internal.h"

#include <algorithm>
#include <cstring>

namespace muca {

template <int MODE>
struct WeightType { using T = float; };
template <>
struct WeightType<kModeProduce> { using T = double; };

__host__ __device__ constexpr size_t align16(size_t b) { return (b + 15) & ~size_t(15); }

// Shared-memory layout of a sweep block: weights | histogram (weight mode) | lattice.
__host__ __device__ inline size_t smem_weights_bytes(int mode, uint32_t N)
{
    return align16((size_t)(N + 1) * (mode == kModeWeight ? 4 : 8));
}
__host__ __device__ inline size_t smem_hist_bytes(int mode, uint32_t N)
{
    return mode == kModeWeight ? align16((size_t)(N + 1) * 4) : 0;
}

struct ChainState {
    int E, EJ, M;
};

// Random numbers of one group of four attempts: one Philox block of the
// acceptance stream (k1) and one of the direction stream (k3) at the same
// counter, as the reference draws them (muca_delta_multigpu.cu:794-797).
struct Group {
    uint32_t r1[4], r3[4];
};

template <int R>
__device__ __forceinline__ Group gen_group(uint32_t cc, uint32_t seed, uint32_t iter, const RoundKeys<R> &k1,
                                           const RoundKeys<R> &k3)
{
    const uint4 a = philox<R>(cc, seed, iter, kCtrTag, k1);
    const uint4 b = philox<R>(cc, seed, iter, kCtrTag, k3);
    Group g;
    g.r1[0] = a.x; g.r1[1] = a.y; g.r1[2] = a.z; g.r1[3] = a.w;
    g.r3[0] = b.x; g.r3[1] = b.y; g.r3[2] = b.z; g.r3[3] = b.w;
    return g;
}

// Prefetched groups: q0 serves the next four attempts, q1 the four after;
// qc is the counter value of q1.  The counter word 0 runs on from the
// thermalisation into the production phase, as in the reference kernel,
// so the queue simply carries over.
struct Queue {
    Group q0, q1;
    uint32_t qc;
};

template <int R>
__device__ __forceinline__ void refill(Queue &Q, uint32_t consumed, uint32_t seed, uint32_t iter,
                                       const RoundKeys<R> &k1, const RoundKeys<R> &k3)
{
    if (consumed == 2) {
        Q.q0 = gen_group<R>(Q.qc + 1u, seed, iter, k1, k3);
        Q.q1 = gen_group<R>(Q.qc + 2u, seed, iter, k1, k3);
        Q.qc += 2u;
    } else {
        Q.q0 = Q.q1;
        Q.q1 = gen_group<R>(Q.qc + 1u, seed, iter, k1, k3);
        Q.qc += 1u;
    }
}

// One full window: the SLOTS same-parity (HALF) sites of word q of row `row`,
// SLOTS consecutive attempts of the sweep.  lat points at this lane's word 0
// (stride cpb).  `eps` bounds |__logf(u) - logf(u)| over every value u that
// u01fixedpt<float> can produce (measured on the device at context creation).
template <int MODE, int R, int SLOTS, int HALF>
__device__ __forceinline__ void window(uint32_t *__restrict__ lat, uint32_t cpb, uint32_t L, uint32_t WPR,
                                       uint32_t row, uint32_t q, bool rec,
                                       const typename WeightType<MODE>::T *__restrict__ wS,
                                       uint32_t *__restrict__ histS, unsigned long long *__restrict__ histG,
                                       ChainState &st, Queue &Q, uint32_t seed, uint32_t iter, const RoundKeys<R> &k1,
                                       const RoundKeys<R> &k3, typename WeightType<MODE>::T eps)
{
    using WT = typename WeightType<MODE>::T;
    constexpr uint32_t M2 = 0x33333333u;
    const uint32_t rup = (row + 1 == L) ? 0u : row + 1;
    const uint32_t rdn = (row == 0) ? L - 1 : row - 1;
    uint32_t *pc = lat + (size_t)(row * WPR + q) * cpb;
    const uint32_t C = *pc;
    const uint32_t U = lat[(size_t)(rup * WPR + q) * cpb];
    const uint32_t D = lat[(size_t)(rdn * WPR + q) * cpb];
    // the one neighbour outside word q: left of the first even site, or
    // right of the last odd site (wrapping along the row)
    uint32_t sq, sb;
    if (HALF == 0) {
        sq = q ? q - 1 : (L - 1) >> 4;
        sb = q ? 15u : ((L - 1) & 15u);
    } else {
        sq = (16 * q + 16 < L) ? q + 1 : 0u;
        sb = 0u;
    }
    const uint32_t sv = spin_code(lat[(size_t)(row * WPR + sq) * cpb], sb);

    // Nibble t of `ctr` holds the spin code of the window's site t; nibble t
    // of `nbs` the sum of its four neighbours' codes (0..8, no carries).
    uint32_t ctr, nbs;
    if (HALF == 0) {
        const uint32_t oc = (C >> 2) & M2;  // odd sites: right neighbours, shifted: left ones
        ctr = C & M2;
        nbs = oc + ((oc << 4) | sv) + (U & M2) + (D & M2);
    } else {
        const uint32_t ec = C & M2;  // even sites: left neighbours, shifted: right ones
        ctr = (C >> 2) & M2;
        nbs = ec + ((ec >> 4) | (sv << (4 * (SLOTS - 1)))) + ((U >> 2) & M2) + ((D >> 2) & M2);
    }

    uint32_t r1[SLOTS], r3[SLOTS];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        r1[t] = Q.q0.r1[t];
        r3[t] = Q.q0.r3[t];
        if (SLOTS == 8) {
            r1[t + 4] = Q.q1.r1[t];
            r3[t + 4] = Q.q1.r3[t];
        }
    }
    // the next window's random numbers: independent of everything below,
    // so they fill the issue slots of the sequential scan
    refill<R>(Q, SLOTS / 4, seed, iter, k1, k3);

    // proposals of the whole window (independent of each other):
    // s -> s +/- 1 with the cyclic wrap is (code + 1 + d) mod 3 on s+1 codes
    int dE[SLOTS], dDel[SLOTS], dM[SLOTS];
    WT f2[SLOTS];
    float lf[SLOTS];
    uint32_t vnib = 0;
#pragma unroll
    for (int t = 0; t < SLOTS; ++t) {
        const uint32_t vo = (ctr >> (4 * t)) & 3u;
        const int nbc = (int)((nbs >> (4 * t)) & 15u);
        const uint32_t x = vo + 1u + (r3[t] >> 31);  // u01f(r3) < 0.5  <=>  r3 < 2^31
        const uint32_t vn = x >= 3u ? x - 3u : x;
        const int dv = (int)vn - (int)vo;
        dE[t] = dv * (4 - nbc);  // -(s_new - s_old) * sum of neighbour spins
        dDel[t] = (int)(vn != 1u) - (int)(vo != 1u);
        dM[t] = dv;
        f2[t] = (WT)(-2 * dE[t]);
        lf[t] = __logf(u01f(r1[t]));
        vnib |= vn << (4 * t);
    }

    // sequential accept/reject over E_Delta:
    //   accept  <=>  diff >= 0  ||  logf(u) < diff,
    //   diff = (float)(-2 dE) + w[E + dDel] - w[E]   (muca_delta_multigpu.cu:810-816)
    // decided with __logf(u) unless it lies within eps of diff in some lane;
    // then the window is replayed with the exact logf(u).
    const ChainState s0 = st;
    const WT wE0 = wS[st.E];
    WT wE = wE0;
    uint32_t accm = 0;
    bool near = false;
    int Es[SLOTS], Ms[SLOTS];
#pragma unroll
    for (int t = 0; t < SLOTS; ++t) {
        const WT wn = wS[st.E + dDel[t]];
        WT diff;
        if (MODE == kModeWeight)
            diff = __fsub_rn(__fadd_rn((float)f2[t], (float)wn), (float)wE);
        else
            diff = __dsub_rn(__dadd_rn((double)f2[t], (double)wn), (double)wE);
        const WT l = (WT)lf[t];
        const bool acc = (diff >= (WT)0) || (l < diff);
        near |= (diff < (WT)0) && (fabs(l - diff) <= eps);
        if (acc) {
            st.E += dDel[t];
            st.EJ += dE[t];
            st.M += dM[t];
            wE = wn;
            accm |= 0xFu << (4 * t);
        }
        Es[t] = st.E;
        Ms[t] = st.M;
    }
    if (__any_sync(0xffffffffu, near)) {
        st = s0;
        wE = wE0;
        accm = 0;
#pragma unroll
        for (int t = 0; t < SLOTS; ++t) {
            const WT wn = wS[st.E + dDel[t]];
            WT diff;
            if (MODE == kModeWeight)
                diff = __fsub_rn(__fadd_rn((float)f2[t], (float)wn), (float)wE);
            else
                diff = __dsub_rn(__dadd_rn((double)f2[t], (double)wn), (double)wE);
            bool acc = diff >= (WT)0;
            if (!acc) acc = (WT)logf(u01f(r1[t])) < diff;
            if (acc) {
                st.E += dDel[t];
                st.EJ += dE[t];
                st.M += dM[t];
                wE = wn;
                accm |= 0xFu << (4 * t);
            }
            Es[t] = st.E;
            Ms[t] = st.M;
        }
    }
    const uint32_t merged = (ctr & ~accm) | (vnib & accm);
    *pc = (HALF == 0) ? ((C & ~M2) | merged) : ((C & M2) | (merged << 2));
    if (rec) {
#pragma unroll
        for (int t = 0; t < SLOTS; ++t) {
            if (MODE == kModeWeight)
                atomicAdd(&histS[Es[t]], 1u);
            else
                atomicAdd(&histG[(uint32_t)(Ms[t] + Es[t] * Es[t] + 2 * Es[t]) >> 1], 1ull);
        }
    }
}

// The first `len` (< cnt) attempts of a window, one at a time as the
// reference writes them; only the last window of a phase can be partial.
template <int MODE, int R>
__device__ __noinline__ void partial_window(uint32_t *__restrict__ lat, uint32_t cpb, uint32_t L, uint32_t WPR,
                                            uint32_t row, uint32_t q, uint32_t half, uint32_t len, bool rec,
                                            const typename WeightType<MODE>::T *__restrict__ wS,
                                            uint32_t *__restrict__ histS, unsigned long long *__restrict__ histG,
                                            ChainState &st, Queue &Q, uint32_t seed, uint32_t iter,
                                            const RoundKeys<R> &k1, const RoundKeys<R> &k3)
{
    using WT = typename WeightType<MODE>::T;
    auto word = [&](uint32_t r, uint32_t c) -> uint32_t * { return lat + (size_t)(r * WPR + (c >> 4)) * cpb; };
    auto get = [&](uint32_t r, uint32_t c) -> int { return (int)spin_code(*word(r, c), c) - 1; };
    const uint32_t rup = (row + 1 == L) ? 0u : row + 1;
    const uint32_t rdn = (row == 0) ? L - 1 : row - 1;
    for (uint32_t t = 0; t < len; ++t) {
        const uint32_t r1 = t < 4 ? Q.q0.r1[t & 3] : Q.q1.r1[t & 3];
        const uint32_t r3 = t < 4 ? Q.q0.r3[t & 3] : Q.q1.r3[t & 3];
        const uint32_t col = 16u * q + 2u * t + half;
        const uint32_t cl = col ? col - 1 : L - 1, cr = (col + 1 == L) ? 0u : col + 1;
        const int os = get(row, col);
        int ns = os + ((r3 >> 31) ? -1 : 1);
        ns = ns - 3 * (ns == 2) + 3 * (ns == -2);
        const int nb = get(row, cl) + get(row, cr) + get(rup, col) + get(rdn, col);
        const int dE = -(ns - os) * nb, dDel = ns * ns - os * os, dM = ns - os;
        WT diff;
        if (MODE == kModeWeight)
            diff = __fsub_rn(__fadd_rn((float)(-2 * dE), (float)wS[st.E + dDel]), (float)wS[st.E]);
        else
            diff = __dsub_rn(__dadd_rn((double)(-2 * dE), (double)wS[st.E + dDel]), (double)wS[st.E]);
        bool acc = diff >= (WT)0;
        if (!acc) acc = (WT)logf(u01f(r1)) < diff;
        if (acc) {
            uint32_t *p = word(row, col);
            const uint32_t sh = 2u * (col & 15u);
            *p = (*p & ~(3u << sh)) | ((uint32_t)(ns + 1) << sh);
            st.E += dDel;
            st.EJ += dE;
            st.M += dM;
        }
        if (rec) {
            if (MODE == kModeWeight)
                atomicAdd(&histS[st.E], 1u);
            else
                atomicAdd(&histG[(uint32_t)(st.M + st.E * st.E + 2 * st.E) >> 1], 1ull);
        }
    }
    refill<R>(Q, (len + 3u) >> 2, seed, iter, k1, k3);
}

template <int MODE>
__device__ __forceinline__ void flush_hist(uint32_t *histS, unsigned long long *histG, uint32_t N)
{
    if (MODE != kModeWeight) return;
    __syncthreads();
    for (uint32_t b = threadIdx.x; b <= N; b += blockDim.x) {
        const uint32_t v = histS[b];
        if (v) {
            atomicAdd(&histG[b], (unsigned long long)v);
            histS[b] = 0;
        }
    }
    __syncthreads();
}

// Common prologue: stage weights / clear histogram / stage lattice.
template <int MODE, bool LAT_SMEM>
__device__ __forceinline__ uint32_t *prologue(const SweepArgs &a, unsigned char *smem,
                                              typename WeightType<MODE>::T *&wS, uint32_t *&histS,
                                              uint32_t *&gl)
{
    using WT = typename WeightType<MODE>::T;
    const uint32_t N = a.N, cpb = blockDim.x, tid = threadIdx.x;
    wS = reinterpret_cast<WT *>(smem);
    histS = reinterpret_cast<uint32_t *>(smem + smem_weights_bytes(MODE, N));
    uint32_t *latS = reinterpret_cast<uint32_t *>(smem + smem_weights_bytes(MODE, N) + smem_hist_bytes(MODE, N));
    const WT *wg = reinterpret_cast<const WT *>(a.w);
    for (uint32_t i = tid; i <= N; i += cpb) wS[i] = wg[i];
    if (MODE == kModeWeight)
        for (uint32_t i = tid; i <= N; i += cpb) histS[i] = 0u;
    const uint32_t words = a.L * a.WPR;
    gl = a.lat + (size_t)blockIdx.x * words * cpb + tid;
    if (LAT_SMEM) {
        for (uint32_t w = 0; w < words; ++w) latS[(size_t)w * cpb + tid] = gl[(size_t)w * cpb];
        return latS + tid;
    }
    return gl;
}

template <int MODE, int R, bool LAT_SMEM>
__global__ void __launch_bounds__(256, 1) k_sweep_fast(const SweepArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    using WT = typename WeightType<MODE>::T;
    uint32_t iter = a.iter;
    unsigned long long therm = a.therm, nup = a.nup;
    if (a.dyn) {
        if (a.dyn[2]) return;
        iter = a.dyn[0];
        nup = a.dyn[1];
    }
    WT *wS;
    uint32_t *histS, *gl;
    uint32_t *lat = prologue<MODE, LAT_SMEM>(a, smem, wS, histS, gl);
    __syncthreads();

    const uint32_t cpb = blockDim.x, tid = threadIdx.x;
    const uint32_t chain = blockIdx.x * cpb + tid;
    const bool active = chain < a.nchains;
    const uint32_t dev = chain / a.chains_per_dev;
    const uint32_t W = chain - dev * a.chains_per_dev;
    const uint32_t seed = a.seed_base + a.seed_dev_mul * dev;
    RoundKeys<R> k1, k3;
    k1.init(a.k1_mul * W + a.k1_add, a.k1_hi);
    k3.init(a.k3_mul * W + a.k3_add, a.k3_hi);
    ChainState st;
    st.E = active ? a.edel[chain] : 0;
    st.EJ = active ? a.ej[chain] : 0;
    st.M = (active && MODE == kModeProduce) ? a.mag[chain] : 0;
    Queue Q;
    Q.q0 = gen_group<R>(1u, seed, iter, k1, k3);
    Q.q1 = gen_group<R>(2u, seed, iter, k1, k3);
    Q.qc = 2u;
    const WT eps = (WT)a.log_eps;
    const uint32_t L = a.L, WPR = a.WPR;
    // a block's u32 histogram bins can take at most 2^31 counts between flushes
    const unsigned long long flush_every = (MODE == kModeWeight) ? (0x80000000ull / cpb) : ~0ull;

    for (int phase = 0; phase < 2; ++phase) {
        const unsigned long long n = phase ? nup : therm;
        const bool rec = phase == 1;
        const bool rec_lane = rec && active;
        unsigned long long i = 0, since_flush = 0;
        uint32_t row = 0, q = 0, half = 0;
        while (i < n) {
            const uint32_t cnt = (min(16u * q + 16u, L) - 16u * q) >> 1;
            if (n - i < cnt) {
                partial_window<MODE, R>(lat, cpb, L, WPR, row, q, half, (uint32_t)(n - i), rec_lane, wS, histS,
                                        a.hist, st, Q, seed, iter, k1, k3);
                break;
            }
            if (cnt == 8) {
                if (half) window<MODE, R, 8, 1>(lat, cpb, L, WPR, row, q, rec_lane, wS, histS, a.hist, st, Q, seed, iter, k1, k3, eps);
                else      window<MODE, R, 8, 0>(lat, cpb, L, WPR, row, q, rec_lane, wS, histS, a.hist, st, Q, seed, iter, k1, k3, eps);
            } else {
                if (half) window<MODE, R, 4, 1>(lat, cpb, L, WPR, row, q, rec_lane, wS, histS, a.hist, st, Q, seed, iter, k1, k3, eps);
                else      window<MODE, R, 4, 0>(lat, cpb, L, WPR, row, q, rec_lane, wS, histS, a.hist, st, Q, seed, iter, k1, k3, eps);
            }
            i += cnt;
            if (++q == WPR) {
                q = 0;
                if (++row == L) { row = 0; half ^= 1u; }
            }
            if (rec) {
                since_flush += cnt;
                if (since_flush >= flush_every && i < n) {
                    flush_hist<MODE>(histS, a.hist, a.N);
                    since_flush = 0;
                }
            }
        }
    }

    if (LAT_SMEM) {
        const uint32_t words = L * WPR;
        for (uint32_t w = 0; w < words; ++w) gl[(size_t)w * cpb] = lat[(size_t)w * cpb];
    }
    if (active) {
        a.edel[chain] = st.E;
        a.ej[chain] = st.EJ;
        if (MODE == kModeProduce) a.mag[chain] = st.M;
    }
    flush_hist<MODE>(histS, a.hist, a.N);
}

template <int MODE, int R, bool LAT_SMEM>
__global__ void __launch_bounds__(256) k_sweep_generic(const SweepArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    using WT = typename WeightType<MODE>::T;
    uint32_t iter = a.iter;
    unsigned long long therm = a.therm, nup = a.nup;
    if (a.dyn) {
        if (a.dyn[2]) return;
        iter = a.dyn[0];
        nup = a.dyn[1];
    }
    WT *wS;
    uint32_t *histS, *gl;
    uint32_t *lat = prologue<MODE, LAT_SMEM>(a, smem, wS, histS, gl);
    __syncthreads();

    const uint32_t cpb = blockDim.x, tid = threadIdx.x;
    const uint32_t chain = blockIdx.x * cpb + tid;
    const bool active = chain < a.nchains;
    const uint32_t dev = chain / a.chains_per_dev;
    const uint32_t W = chain - dev * a.chains_per_dev;
    const uint32_t seed = a.seed_base + a.seed_dev_mul * dev;
    RoundKeys<R> k1, k3;
    k1.init(a.k1_mul * W + a.k1_add, a.k1_hi);
    k3.init(a.k3_mul * W + a.k3_add, a.k3_hi);
    int E = active ? a.edel[chain] : 0;
    int EJ = active ? a.ej[chain] : 0;
    int M = (active && MODE == kModeProduce) ? a.mag[chain] : 0;
    uint32_t c0 = 0;
    const uint32_t L = a.L, N = a.N, WPR = a.WPR;
    uint4 r1 = make_uint4(0, 0, 0, 0), r3 = r1;
    const unsigned long long flush_every = (MODE == kModeWeight) ? (0x80000000ull / cpb) : ~0ull;
    auto word_of = [&](uint32_t site) -> uint32_t * {
        const uint32_t r = site / L, c = site - r * L;
        return lat + (size_t)(r * WPR + (c >> 4)) * cpb;
    };
    auto get = [&](uint32_t site) -> int {
        const uint32_t c = site % L;
        return (int)spin_code(*word_of(site), c) - 1;
    };
    auto put = [&](uint32_t site, int s) {
        const uint32_t c = site % L;
        uint32_t *p = word_of(site);
        const uint32_t sh = 2u * (c & 15u);
        *p = (*p & ~(3u << sh)) | ((uint32_t)(s + 1) << sh);
    };
    for (int phase = 0; phase < 2; ++phase) {
        const unsigned long long n = phase ? nup : therm;
        unsigned long long since_flush = 0;
        for (unsigned long long i = 0; i < n; ++i) {
            if ((i & 3ull) == 0) {
                ++c0;
                r1 = philox<R>(c0, seed, iter, kCtrTag, k1);
                r3 = philox<R>(c0, seed, iter, kCtrTag, k3);
            }
            const int sub = (int)(i & 3ull);
            const uint32_t idx = a.index[i % N];
            int ns = get(idx) + 2 * (u01f(pick(r3, sub)) < 0.5f) - 1;
            const int os = get(idx);
            ns = ns - 3 * (ns == 2) + 3 * (ns == -2);
            put(idx, ns * (os == 0) + os);
            const int dE = ((os == 0) + os * (ns - os)) * (-get(idx)) *
                           (get(a.naver[4 * idx]) + get(a.naver[4 * idx + 1]) + get(a.naver[4 * idx + 2]) +
                            get(a.naver[4 * idx + 3]));
            const int dDel = ns * ns - os * os, dM = ns - os;
            WT diff;
            if (MODE == kModeWeight)
                diff = __fsub_rn(__fadd_rn((float)(-dE * 2), (float)wS[E + dDel]), (float)wS[E]);
            else
                diff = __dsub_rn(__dadd_rn((double)(-dE * 2), (double)wS[E + dDel]), (double)wS[E]);
            bool acc = diff >= (WT)0;
            if (!acc) acc = (WT)logf(u01f(pick(r1, sub))) < diff;
            if (acc) {
                put(idx, ns);
                EJ += dE;
                E += dDel;
                M += dM;
            } else {
                put(idx, os);
            }
            if (phase == 1) {
                if (active) {
                    if (MODE == kModeWeight) atomicAdd(&histS[E], 1u);
                    else atomicAdd(&a.hist[(uint32_t)(M + E * E + 2 * E) >> 1], 1ull);
                }
                if (++since_flush >= flush_every && i + 1 < n) {
                    flush_hist<MODE>(histS, a.hist, N);
                    since_flush = 0;
                }
            }
        }
    }
    if (LAT_SMEM) {
        const uint32_t words = L * WPR;
        for (uint32_t w = 0; w < words; ++w) gl[(size_t)w * cpb] = lat[(size_t)w * cpb];
    }
    if (active) {
        a.edel[chain] = E;
        a.ej[chain] = EJ;
        if (MODE == kModeProduce) a.mag[chain] = M;
    }
    flush_hist<MODE>(histS, a.hist, N);
}

// ---------------------------------------------------------------------------
// Worst-case |__logf(u) - logf(u)| over every value u01fixedpt<float> can
// return (u = (2k+1) 2^-24, k < 2^23), as the bits of a non-negative float.
__global__ void k_logf_bracket(unsigned int *maxbits)
{
    unsigned int m = 0;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < (1u << 23); k += gridDim.x * blockDim.x) {
        const float u = u01f(k << 9);
        const float e = fabsf(__logf(u) - logf(u));
        m = max(m, __float_as_uint(e));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxbits, m);
}

cudaError_t measure_logf_bracket(float *max_abs_err, cudaStream_t s)
{
    unsigned int *d = nullptr, h = 0;
    cudaError_t e = cudaMalloc(&d, sizeof(unsigned int));
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(d, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) {
        k_logf_bracket<<<152 * 8, 256, 0, s>>>(d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof h, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d);
    float f;
    std::memcpy(&f, &h, sizeof f);
    *max_abs_err = f;
    return e;
}

SweepPlan plan_sweep(int mode, int rounds, uint32_t L, uint32_t nchains, size_t smem_optin, int sms)
{
    SweepPlan p{};
    p.mode = mode;
    p.rounds = rounds;
    p.fast = (L % 8 == 0) && L >= 8;
    const uint32_t N = L * L, WPR = (L + 15) / 16;
    const size_t fixed = smem_weights_bytes(mode, N) + smem_hist_bytes(mode, N);
    const size_t per_chain = (size_t)L * WPR * 4;
    // Chains per block: one block per SM holding a multiple of 32 chains,
    // spread over the SMs; capped by shared memory when the lattice is staged.
    uint32_t per_sm = (nchains + (uint32_t)sms - 1) / (uint32_t)sms;
    uint32_t cpb = std::max<uint32_t>(32u, std::min<uint32_t>(256u, (per_sm + 31u) / 32u * 32u));
    size_t cap = smem_optin > fixed ? (smem_optin - fixed) / per_chain : 0;
    uint32_t cap32 = (uint32_t)std::min<size_t>(256, cap / 32 * 32);
    if (cap32 >= 32) {
        p.lat_smem = true;
        cpb = std::min(cpb, cap32);
    } else {
        p.lat_smem = false;
    }
    p.cpb = cpb;
    p.blocks = (nchains + cpb - 1) / cpb;
    p.smem = fixed + (p.lat_smem ? per_chain * cpb : 0);
    return p;
}

template <int MODE, int R, bool LS>
static cudaError_t launch_one(const SweepPlan &p, const SweepArgs &a, cudaStream_t s)
{
    auto kern = p.fast ? k_sweep_fast<MODE, R, LS> : k_sweep_generic<MODE, R, LS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem);
    if (e != cudaSuccess) return e;
    kern<<<p.blocks, p.cpb, p.smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_sweep(const SweepPlan &p, const SweepArgs &a, cudaStream_t s)
{
#define MUCA_DISPATCH(M, R)                                                          \
    return p.lat_smem ? launch_one<M, R, true>(p, a, s) : launch_one<M, R, false>(p, a, s)
    if (p.mode == kModeWeight) {
        if (p.rounds == 10) MUCA_DISPATCH(kModeWeight, 10);
        MUCA_DISPATCH(kModeWeight, 7);
    } else {
        if (p.rounds == 10) MUCA_DISPATCH(kModeProduce, 10);
        MUCA_DISPATCH(kModeProduce, 7);
    }
#undef MUCA_DISPATCH
}

}  // namespace muca
