// k_sweep.cu -- Metropolis sweep kernels of the multicanonical hot path.
//
// One chain per lane, as in the reference kernels mcs
// (muca_delta_multigpu.cu:737-829, weight estimation, FP32 weights, 1D
// histogram of E_Delta) and mcs (produce2_multigpu.cu:401-496, production,
// FP64 weights, M tracked, 2D (E_Delta, M) histogram).  Every attempt
// reproduces the reference's arithmetic: same Philox4x32 keys and counters,
// same sweep order (even linear sites, then odd ones: :173), same proposal
// (s -> s +/- 1 with the cyclic wrap of :802), same
//   diff = (float)(-2 dE) + w[E + dDel] - w[E]        (:810)
// evaluated without contraction, and the same test diff >= 0 || logf(u) < diff.
//
// GB300 layout (windowed kernels, L % 8 == 0):
//   * the lattice lives in shared memory, 2 bits per spin, rows padded to
//     16-site words, [word][lane] so the lanes of a warp hit distinct banks;
//   * the weights (FP32 or FP64) and, in weight mode, a u32 histogram live in
//     shared memory; the histogram is drained to the u64 device histogram
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
//     lane, so every decision equals the reference's logf decision.
// Kernels:
//   k_sweep_spec  warp-specialised: per 32 chains one producer warp draws the
//                 Philox numbers (two blocks per four attempts) into a
//                 4-deep shared-memory ring guarded by mbarriers, and one
//                 consumer warp runs decode, scan, write-back and histogram;
//                 the producer's integer work fills the consumer's latency;
//   k_sweep_win   the same window core with the Philox numbers drawn by the
//                 chain's own lane, one window ahead;
//   k_sweep_generic  the reference step by step on the packed layout, any L.
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

// Shared-memory layout: weights | histogram (weight mode) | ring + barriers (specialised) | lattice.
__host__ __device__ inline size_t smem_weights_bytes(int mode, uint32_t N)
{
    return align16((size_t)(N + 1) * (mode == kModeWeight ? 4 : 8));
}
__host__ __device__ inline size_t smem_hist_bytes(int mode, uint32_t N)
{
    return mode == kModeWeight ? align16((size_t)(N + 1) * 4) : 0;
}
// ring: [pair][depth][slot 0..7][lane 0..31] u32, then full/empty mbarriers
__host__ __device__ inline size_t smem_ring_bytes(uint32_t pairs)
{
    return (size_t)pairs * kRingDepth * 8 * 32 * 4 + (size_t)pairs * kRingDepth * 2 * 8;
}

struct ChainState {
    int E, EJ, M;
};

// A packed random word per attempt: bits 31..8 are the top 24 bits of the
// acceptance draw r1 (all that u01fixedpt<float> uses: u = (1|(r1>>8))
// 2^-24), bit 0 is the direction bit (u01fixedpt<float>(r3) < 0.5 <=>
// r3 < 2^31, so the bit is r3's top bit, set for s -> s-1).
__device__ __forceinline__ uint32_t pack_draw(uint32_t r1, uint32_t r3) { return (r1 & 0xFFFFFF00u) | (r3 >> 31); }

template <int R>
__device__ __forceinline__ void draw_group(uint32_t cc, uint32_t seed, uint32_t iter, const RoundKeys<R> &k1,
                                           const RoundKeys<R> &k3, uint32_t *p)
{
    // one Philox block of the acceptance stream (k1) and one of the direction
    // stream (k3) at the same counter (muca_delta_multigpu.cu:794-797)
    const uint4 a = philox<R>(cc, seed, iter, kCtrTag, k1);
    const uint4 b = philox<R>(cc, seed, iter, kCtrTag, k3);
    p[0] = pack_draw(a.x, b.x);
    p[1] = pack_draw(a.y, b.y);
    p[2] = pack_draw(a.z, b.z);
    p[3] = pack_draw(a.w, b.w);
}

// Histogram entry.  The u32 shared bins are drained into the u64 device
// histogram by the lane whose increment finds 2^31 counts already there.
template <int MODE>
__device__ __forceinline__ void record(uint32_t *histS, unsigned long long *histG, int E, int M)
{
    if (MODE == kModeWeight) {
        const uint32_t old = atomicAdd(&histS[E], 1u);
        if (old >= 0x80000000u) {
            const uint32_t v = atomicExch(&histS[E], 0u);
            atomicAdd(&histG[E], (unsigned long long)v);
        }
    } else {
        atomicAdd(&histG[(uint32_t)(M + E * E + 2 * E) >> 1], 1ull);
    }
}

// Histogram entries of one window, merged into runs of equal bins per lane
// (E_Delta moves by at most one per attempt, so a window's entries cluster).
// `checked` (uniform: the launch can put 2^32 entries into one block's bins)
// drains a u32 shared bin into the u64 device histogram once it holds 2^31.
template <int MODE, int SLOTS>
__device__ __forceinline__ void record_window(uint32_t *__restrict__ histS, unsigned long long *__restrict__ histG,
                                              const int (&Es)[SLOTS], const int (&Ms)[SLOTS], bool checked)
{
    if (MODE == kModeWeight) {
        if (checked) {
#pragma unroll
            for (int t = 0; t < SLOTS; ++t) {
                const uint32_t old = atomicAdd(&histS[Es[t]], 1u);
                if (old >= 0x80000000u) atomicAdd(&histG[Es[t]], (unsigned long long)atomicExch(&histS[Es[t]], 0u));
            }
            return;
        }
        int cur = Es[0];
        uint32_t cnt = 1;
#pragma unroll
        for (int t = 1; t < SLOTS; ++t) {
            const bool same = Es[t] == cur;
            if (!same) atomicAdd(&histS[cur], cnt);
            cnt = same ? cnt + 1u : 1u;
            cur = Es[t];
        }
        atomicAdd(&histS[cur], cnt);
    } else {
        uint32_t cur = (uint32_t)(Ms[0] + Es[0] * Es[0] + 2 * Es[0]) >> 1;
        unsigned long long cnt = 1;
#pragma unroll
        for (int t = 1; t < SLOTS; ++t) {
            const uint32_t b = (uint32_t)(Ms[t] + Es[t] * Es[t] + 2 * Es[t]) >> 1;
            const bool same = b == cur;
            if (!same) atomicAdd(&histG[cur], cnt);
            cnt = same ? cnt + 1ull : 1ull;
            cur = b;
        }
        atomicAdd(&histG[cur], cnt);
    }
}

// One full window: the SLOTS same-parity (HALF) sites of word q of row `row`,
// SLOTS consecutive attempts of the sweep, with packed draws p[].  lat points
// at this lane's word 0 (stride cpb).  `store` is false for padding lanes:
// they read another lane's spins, never accept (so their E stays at 2 and
// every weight index E + dDel_t + dDel_t+1 stays in [0, 4]) and never write.
template <int MODE, int SLOTS, int HALF>
__device__ __forceinline__ void window_core(uint32_t *__restrict__ lat, uint32_t cpb, uint32_t L, uint32_t WPR,
                                            uint32_t row, uint32_t q, bool rec, bool store, bool checked,
                                            const typename WeightType<MODE>::T *__restrict__ wS,
                                            uint32_t *__restrict__ histS, unsigned long long *__restrict__ histG,
                                            ChainState &st, const uint32_t (&p)[SLOTS],
                                            typename WeightType<MODE>::T eps)
{
    using WT = typename WeightType<MODE>::T;
    constexpr uint32_t M2 = 0x33333333u, N1 = 0x11111111u;
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

    // Nibble t of `ctr` holds the spin code (s+1) of the window's site t;
    // nibble t of `nbs` the sum of its four neighbours' codes (0..8, no carries).
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
    // Proposals of all sites at once, nibble-parallel:  s -> s +/- 1 with the
    // cyclic wrap is code -> (code + 1 + d) mod 3, d the direction bit.
    uint32_t dn = 0;
#pragma unroll
    for (int t = 0; t < SLOTS; ++t) dn |= (p[t] & 1u) << (4 * t);
    const uint32_t x = ctr + N1 + dn;                              // 1..4
    const uint32_t ge3 = ((x + N1) >> 2) & N1;                     // 1 where x >= 3
    const uint32_t vnib = x - (ge3 + (ge3 << 1));                  // new codes 0..2
    const uint32_t nzo = ((ctr ^ N1) | ((ctr ^ N1) >> 1)) & N1;    // s_old != 0
    const uint32_t nzn = ((vnib ^ N1) | ((vnib ^ N1) >> 1)) & N1;  // s_new != 0
    const uint32_t ddb = nzn + N1 - nzo;                           // dDel + 1 (0..2)
    const uint32_t dvb = vnib + 0x22222222u - ctr;                 // s_new - s_old + 2 (0..4)

    int dE[SLOTS], dDel[SLOTS], dM[SLOTS];
    WT f2[SLOTS];
    float lf[SLOTS];
#pragma unroll
    for (int t = 0; t < SLOTS; ++t) {
        const int dv = (int)((dvb >> (4 * t)) & 7u) - 2;
        dDel[t] = (int)((ddb >> (4 * t)) & 3u) - 1;
        dE[t] = dv * (4 - (int)((nbs >> (4 * t)) & 15u));  // -(s_new - s_old) * (sum of neighbour spins)
        dM[t] = dv;
        f2[t] = (WT)(-2 * dE[t]);
        lf[t] = __logf(u01f(p[t]));
    }

    // Sequential accept/reject over E_Delta:
    //   accept  <=>  diff >= 0  ||  logf(u) < diff,
    //   diff = (float)(-2 dE) + w[E + dDel] - w[E]   (muca_delta_multigpu.cu:810-816)
    // decided with __logf(u) unless it lies within eps of diff in some lane;
    // then the window is replayed with the exact logf(u).  The weight of the
    // next attempt is fetched one attempt ahead for both outcomes (c0: this
    // attempt rejected, c1: accepted), so no shared-memory load sits on the
    // dependency chain from one decision to the next.
    const ChainState s0 = st;
    const WT wE0 = wS[st.E];
    WT wE = wE0;
    WT A = wS[st.E + dDel[0]];
    WT c0 = A, c1 = A;
    if (SLOTS > 1) {
        c0 = wS[st.E + dDel[1]];
        c1 = wS[st.E + dDel[0] + dDel[1]];
    }
    uint32_t accm = 0;
    bool near = false;
    int Es[SLOTS], Ms[SLOTS];
#pragma unroll
    for (int t = 0; t < SLOTS; ++t) {
        WT diff;
        if (MODE == kModeWeight)
            diff = __fsub_rn(__fadd_rn((float)f2[t], (float)A), (float)wE);
        else
            diff = __dsub_rn(__dadd_rn((double)f2[t], (double)A), (double)wE);
        const WT l = (WT)lf[t];
        const bool acc = store && ((diff >= (WT)0) || (l < diff));
        near |= (diff < (WT)0) && (fabs(l - diff) <= eps);
        if (acc) {
            st.E += dDel[t];
            st.EJ += dE[t];
            st.M += dM[t];
            wE = A;
            accm |= 0xFu << (4 * t);
        }
        Es[t] = st.E;
        Ms[t] = st.M;
        if (t + 1 < SLOTS) {
            A = acc ? c1 : c0;
            if (t + 2 < SLOTS) {
                c0 = wS[st.E + dDel[t + 2]];
                c1 = wS[st.E + dDel[t + 1] + dDel[t + 2]];
            }
        }
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
            if (!acc) acc = (WT)logf(u01f(p[t])) < diff;
            acc = acc && store;
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
    if (store) *pc = (HALF == 0) ? ((C & ~M2) | merged) : ((C & M2) | (merged << 2));
    if (rec) record_window<MODE, SLOTS>(histS, histG, Es, Ms, checked);
}

// The first `len` (< window size) attempts of a window, one at a time as
// the reference writes them; only the last window of a phase is partial.
template <int MODE>
__device__ __noinline__ void partial_core(uint32_t *__restrict__ lat, uint32_t cpb, uint32_t L, uint32_t WPR,
                                          uint32_t row, uint32_t q, uint32_t half, uint32_t len, bool rec,
                                          bool store, const typename WeightType<MODE>::T *__restrict__ wS,
                                          uint32_t *__restrict__ histS, unsigned long long *__restrict__ histG,
                                          ChainState &st, const uint32_t *p)
{
    using WT = typename WeightType<MODE>::T;
    const uint32_t rup = (row + 1 == L) ? 0u : row + 1;
    const uint32_t rdn = (row == 0) ? L - 1 : row - 1;
    for (uint32_t t = 0; t < len; ++t) {
        const uint32_t col = 16u * q + 2u * t + half;
        const uint32_t cl = col ? col - 1 : L - 1, cr = (col + 1 == L) ? 0u : col + 1;
        uint32_t *pw = lat + (size_t)(row * WPR + (col >> 4)) * cpb;
        const int os = (int)spin_code(*pw, col) - 1;
        int ns = os + ((p[t] & 1u) ? -1 : 1);
        ns = ns - 3 * (ns == 2) + 3 * (ns == -2);
        const int nb = (int)spin_code(lat[(size_t)(row * WPR + (cl >> 4)) * cpb], cl) +
                       (int)spin_code(lat[(size_t)(row * WPR + (cr >> 4)) * cpb], cr) +
                       (int)spin_code(lat[(size_t)(rup * WPR + (col >> 4)) * cpb], col) +
                       (int)spin_code(lat[(size_t)(rdn * WPR + (col >> 4)) * cpb], col) - 4;
        const int dE = -(ns - os) * nb, dDel = ns * ns - os * os, dM = ns - os;
        WT diff;
        if (MODE == kModeWeight)
            diff = __fsub_rn(__fadd_rn((float)(-2 * dE), (float)wS[st.E + dDel]), (float)wS[st.E]);
        else
            diff = __dsub_rn(__dadd_rn((double)(-2 * dE), (double)wS[st.E + dDel]), (double)wS[st.E]);
        bool acc = diff >= (WT)0;
        if (!acc) acc = (WT)logf(u01f(p[t])) < diff;
        if (acc && store) {
            const uint32_t sh = 2u * (col & 15u);
            *pw = (*pw & ~(3u << sh)) | ((uint32_t)(ns + 1) << sh);
            st.E += dDel;
            st.EJ += dE;
            st.M += dM;
        }
        if (rec) record<MODE>(histS, histG, st.E, st.M);
    }
}

// Stage weights, clear the histogram, stage this block's lattice; returns
// the lane's lattice base (shared or global).  Only lanes < cpb copy.
template <int MODE, bool LAT_SMEM>
__device__ __forceinline__ uint32_t *prologue(const SweepArgs &a, unsigned char *smem, size_t lat_offset,
                                              uint32_t cpb, uint32_t lane, typename WeightType<MODE>::T *&wS,
                                              uint32_t *&histS, uint32_t *&gl)
{
    using WT = typename WeightType<MODE>::T;
    const uint32_t N = a.N, nt = blockDim.x, tid = threadIdx.x;
    wS = reinterpret_cast<WT *>(smem);
    histS = reinterpret_cast<uint32_t *>(smem + smem_weights_bytes(MODE, N));
    uint32_t *latS = reinterpret_cast<uint32_t *>(smem + lat_offset);
    const WT *wg = reinterpret_cast<const WT *>(a.w);
    for (uint32_t i = tid; i <= N; i += nt) wS[i] = wg[i];
    if (MODE == kModeWeight)
        for (uint32_t i = tid; i <= N; i += nt) histS[i] = 0u;
    const uint32_t words = a.L * a.WPR;
    const uint32_t l = lane < cpb ? lane : 0u;  // padding lanes read lane 0's words, never write
    gl = a.lat + (size_t)blockIdx.x * words * cpb + l;
    if (LAT_SMEM) {
        if (lane < cpb)
            for (uint32_t w = 0; w < words; ++w) latS[(size_t)w * cpb + lane] = gl[(size_t)w * cpb];
        return latS + l;
    }
    return gl;
}

template <int MODE>
__device__ __forceinline__ void drain_hist(uint32_t *histS, unsigned long long *histG, uint32_t N)
{
    if (MODE == kModeWeight) {
        for (uint32_t b = threadIdx.x; b <= N; b += blockDim.x) {
            const uint32_t v = histS[b];
            if (v) atomicAdd(&histG[b], (unsigned long long)v);
        }
    }
}

// Walks the window sequence of a launch: phase 0 (therm) then phase 1 (nup),
// each starting at site 0 of the sweep; calls f(row, q, half, cnt, len, rec)
// and stops early when f returns false.
template <typename F>
__device__ __forceinline__ void for_each_window(uint32_t L, uint32_t WPR, unsigned long long therm,
                                                unsigned long long nup, F &&f)
{
    for (int phase = 0; phase < 2; ++phase) {
        const unsigned long long n = phase ? nup : therm;
        unsigned long long i = 0;
        uint32_t row = 0, q = 0, half = 0;
        while (i < n) {
            const uint32_t cnt = (min(16u * q + 16u, L) - 16u * q) >> 1;
            const uint32_t len = (n - i < cnt) ? (uint32_t)(n - i) : cnt;
            if (!f(row, q, half, cnt, len, phase == 1)) return;
            i += len;
            if (++q == WPR) {
                q = 0;
                if (++row == L) { row = 0; half ^= 1u; }
            }
        }
    }
}

template <int MODE, int R>
struct ChainSetup {
    uint32_t chain, seed;
    bool active;
    RoundKeys<R> k1, k3;
    __device__ __forceinline__ void init(const SweepArgs &a, uint32_t cpb, uint32_t lane)
    {
        chain = blockIdx.x * cpb + lane;
        active = lane < cpb && chain < a.nchains;
        const uint32_t dev = chain / a.chains_per_dev;
        const uint32_t W = chain - dev * a.chains_per_dev;
        seed = a.seed_base + a.seed_dev_mul * dev;
        k1.init(a.k1_mul * W + a.k1_add, a.k1_hi);
        k3.init(a.k3_mul * W + a.k3_add, a.k3_hi);
    }
};

__device__ __forceinline__ bool launch_params(const SweepArgs &a, uint32_t &iter, unsigned long long &nup)
{
    iter = a.iter;
    nup = a.nup;
    if (a.dyn) {
        if (a.dyn[2]) return false;
        iter = a.dyn[0];
        nup = a.dyn[1];
    }
    return true;
}

// ---------------------------------------------------------------------------
// Windowed kernel: every lane draws its own Philox numbers one window ahead
// (`next` holds the packed draws of the next two groups, counters cc-1, cc).
// blockDim = cpb rounded up to a warp; lanes >= cpb are padding.
template <int MODE, int R, bool LAT_SMEM>
__global__ void __launch_bounds__(256, 1) k_sweep_win(const SweepArgs a, uint32_t cpb)
{
    extern __shared__ __align__(16) unsigned char smem[];
    using WT = typename WeightType<MODE>::T;
    uint32_t iter;
    unsigned long long nup;
    if (!launch_params(a, iter, nup)) return;
    const uint32_t lane = threadIdx.x;
    WT *wS;
    uint32_t *histS, *gl;
    const size_t lat_off = smem_weights_bytes(MODE, a.N) + smem_hist_bytes(MODE, a.N);
    uint32_t *lat = prologue<MODE, LAT_SMEM>(a, smem, lat_off, cpb, lane, wS, histS, gl);
    __syncthreads();
    ChainSetup<MODE, R> cs;
    cs.init(a, cpb, lane);
    const bool store = lane < cpb;
    ChainState st;
    st.E = cs.active ? a.edel[cs.chain] : (store ? 0 : 2);
    st.EJ = cs.active ? a.ej[cs.chain] : 0;
    st.M = (cs.active && MODE == kModeProduce) ? a.mag[cs.chain] : 0;
    const WT eps = (WT)a.log_eps;
    // u32 shared bins can overflow only if the launch can record 2^32 entries in one block
    const bool checked = (unsigned long long)cpb * nup >= 0xFFFFFFFFull;
    const uint32_t L = a.L, WPR = a.WPR;
    uint32_t next[8];
    draw_group<R>(1u, cs.seed, iter, cs.k1, cs.k3, next);
    draw_group<R>(2u, cs.seed, iter, cs.k1, cs.k3, next + 4);
    uint32_t cc = 2;
    auto advance = [&](uint32_t groups) {
        if (groups == 2) {
            draw_group<R>(cc + 1, cs.seed, iter, cs.k1, cs.k3, next);
            draw_group<R>(cc + 2, cs.seed, iter, cs.k1, cs.k3, next + 4);
            cc += 2;
        } else {
#pragma unroll
            for (int t = 0; t < 4; ++t) next[t] = next[t + 4];
            draw_group<R>(cc + 1, cs.seed, iter, cs.k1, cs.k3, next + 4);
            cc += 1;
        }
    };
    for_each_window(L, WPR, a.therm, nup, [&](uint32_t row, uint32_t q, uint32_t half, uint32_t cnt, uint32_t len,
                                              bool rec_phase) {
        const bool rec = rec_phase && cs.active;
        if (len < cnt) {
            partial_core<MODE>(lat, cpb, L, WPR, row, q, half, len, rec, store, wS, histS, a.hist, st, next);
            advance((len + 3u) >> 2);
        } else if (cnt == 8) {
            uint32_t p[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) p[t] = next[t];
            advance(2);  // independent of the window below: overlaps its scan
            if (half) window_core<MODE, 8, 1>(lat, cpb, L, WPR, row, q, rec, store, checked, wS, histS, a.hist, st, p, eps);
            else      window_core<MODE, 8, 0>(lat, cpb, L, WPR, row, q, rec, store, checked, wS, histS, a.hist, st, p, eps);
        } else {
            uint32_t p[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) p[t] = next[t];
            advance(1);
            if (half) window_core<MODE, 4, 1>(lat, cpb, L, WPR, row, q, rec, store, checked, wS, histS, a.hist, st, p, eps);
            else      window_core<MODE, 4, 0>(lat, cpb, L, WPR, row, q, rec, store, checked, wS, histS, a.hist, st, p, eps);
        }
        return true;
    });
    if (LAT_SMEM && store) {
        const uint32_t words = L * WPR;
        for (uint32_t w = 0; w < words; ++w) gl[(size_t)w * cpb] = lat[(size_t)w * cpb];
    }
    if (cs.active) {
        a.edel[cs.chain] = st.E;
        a.ej[cs.chain] = st.EJ;
        if (MODE == kModeProduce) a.mag[cs.chain] = st.M;
    }
    __syncthreads();
    drain_hist<MODE>(histS, a.hist, a.N);
}

// ---------------------------------------------------------------------------
// Warp-specialised kernel.  Warps [0, P) consume, warps [P, 2P) produce; the
// pair (c, P+c) serves the 32 chain slots 32c..32c+31 of the block.
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up (returns false) once clock64() passes `deadline`.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long deadline)
{
    while (!mbar_try_wait(bar, parity))
        if (clock64() > deadline) return false;
    return true;
}

constexpr long long kWaitCycles = 1ll << 34;  // ~8 s at 2 GHz; a normal launch takes milliseconds

template <int MODE, int R, bool LAT_SMEM>
__global__ void __launch_bounds__(256, 1) k_sweep_spec(const SweepArgs a, uint32_t cpb)
{
    extern __shared__ __align__(16) unsigned char smem[];
    using WT = typename WeightType<MODE>::T;
    uint32_t iter;
    unsigned long long nup;
    if (!launch_params(a, iter, nup)) return;
    const uint32_t P = blockDim.x >> 6;  // pairs of warps
    const uint32_t warp = threadIdx.x >> 5, l32 = threadIdx.x & 31u;
    const bool producer = warp >= P;
    const uint32_t pair = producer ? warp - P : warp;
    const uint32_t lane = pair * 32u + l32;  // chain slot in the block
    const size_t ring_off = smem_weights_bytes(MODE, a.N) + smem_hist_bytes(MODE, a.N);
    uint32_t *ring = reinterpret_cast<uint32_t *>(smem + ring_off);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + ring_off + (size_t)P * kRingDepth * 8 * 32 * 4);
    uint64_t *full = bars + (size_t)pair * kRingDepth * 2;
    uint64_t *empty = full + kRingDepth;
    uint32_t *myring = ring + (size_t)pair * kRingDepth * 8 * 32 + l32;
    if (threadIdx.x == 0) {
        for (uint32_t i = 0; i < P * kRingDepth * 2; ++i) mbar_init(bars + i, 32);
    }
    WT *wS;
    uint32_t *histS, *gl;
    const size_t lat_off = ring_off + smem_ring_bytes(P);
    uint32_t *lat = prologue<MODE, LAT_SMEM>(a, smem, lat_off, cpb, producer ? 0xFFFFFFFFu : lane, wS, histS, gl);
    __syncthreads();
    ChainSetup<MODE, R> cs;
    cs.init(a, cpb, lane);
    const uint32_t L = a.L, WPR = a.WPR;
    const long long deadline = clock64() + kWaitCycles;
    uint32_t w = 0;  // window counter (ring position)
    bool ok = true;

    if (producer) {
        uint32_t cc = 0;  // Philox counter word 0 of the last drawn group
        for_each_window(L, WPR, a.therm, nup, [&](uint32_t, uint32_t, uint32_t, uint32_t, uint32_t len, bool) {
            const uint32_t s = w % kRingDepth, round = w / kRingDepth;
            uint32_t p[8];
            draw_group<R>(cc + 1, cs.seed, iter, cs.k1, cs.k3, p);
            if (len > 4) draw_group<R>(cc + 2, cs.seed, iter, cs.k1, cs.k3, p + 4);
            cc += (len + 3u) >> 2;
            if (!mbar_wait(empty + s, (round & 1u) ^ 1u, deadline)) { ok = false; return false; }
            uint32_t *slot = myring + (size_t)s * 8 * 32;
#pragma unroll
            for (int t = 0; t < 8; ++t) slot[t * 32] = p[t];
            mbar_arrive(full + s);
            ++w;
            return true;
        });
    } else {
        const bool store = lane < cpb;
        ChainState st;
        st.E = cs.active ? a.edel[cs.chain] : (store ? 0 : 2);
        st.EJ = cs.active ? a.ej[cs.chain] : 0;
        st.M = (cs.active && MODE == kModeProduce) ? a.mag[cs.chain] : 0;
        const WT eps = (WT)a.log_eps;
        const bool checked = (unsigned long long)cpb * nup >= 0xFFFFFFFFull;
        for_each_window(L, WPR, a.therm, nup, [&](uint32_t row, uint32_t q, uint32_t half, uint32_t cnt,
                                                  uint32_t len, bool rec_phase) {
            const uint32_t s = w % kRingDepth, round = w / kRingDepth;
            if (!mbar_wait(full + s, round & 1u, deadline)) { ok = false; return false; }
            const uint32_t *slot = myring + (size_t)s * 8 * 32;
            const bool rec = rec_phase && cs.active;
            if (len < cnt) {
                uint32_t p[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) p[t] = slot[t * 32];
                mbar_arrive(empty + s);
                partial_core<MODE>(lat, cpb, L, WPR, row, q, half, len, rec, store, wS, histS, a.hist, st, p);
            } else if (cnt == 8) {
                uint32_t p[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) p[t] = slot[t * 32];
                mbar_arrive(empty + s);
                if (half) window_core<MODE, 8, 1>(lat, cpb, L, WPR, row, q, rec, store, checked, wS, histS, a.hist, st, p, eps);
                else      window_core<MODE, 8, 0>(lat, cpb, L, WPR, row, q, rec, store, checked, wS, histS, a.hist, st, p, eps);
            } else {
                uint32_t p[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) p[t] = slot[t * 32];
                mbar_arrive(empty + s);
                if (half) window_core<MODE, 4, 1>(lat, cpb, L, WPR, row, q, rec, store, checked, wS, histS, a.hist, st, p, eps);
                else      window_core<MODE, 4, 0>(lat, cpb, L, WPR, row, q, rec, store, checked, wS, histS, a.hist, st, p, eps);
            }
            ++w;
            return true;
        });
        if (LAT_SMEM && store) {
            const uint32_t words = L * WPR;
            for (uint32_t i = 0; i < words; ++i) gl[(size_t)i * cpb] = lat[(size_t)i * cpb];
        }
        if (cs.active && ok) {
            a.edel[cs.chain] = st.E;
            a.ej[cs.chain] = st.EJ;
            if (MODE == kModeProduce) a.mag[cs.chain] = st.M;
        }
    }
    if (!ok && a.err) atomicOr(a.err, 1u);
    __syncthreads();
    drain_hist<MODE>(histS, a.hist, a.N);
}

// ---------------------------------------------------------------------------
// Generic kernel: the reference step as written, for any L, on the packed
// layout; sweep order and neighbours from the reference tables.
template <int MODE, int R, bool LAT_SMEM>
__global__ void __launch_bounds__(256) k_sweep_generic(const SweepArgs a, uint32_t cpb)
{
    extern __shared__ __align__(16) unsigned char smem[];
    using WT = typename WeightType<MODE>::T;
    uint32_t iter;
    unsigned long long nup;
    if (!launch_params(a, iter, nup)) return;
    const uint32_t lane = threadIdx.x;
    WT *wS;
    uint32_t *histS, *gl;
    const size_t lat_off = smem_weights_bytes(MODE, a.N) + smem_hist_bytes(MODE, a.N);
    uint32_t *lat = prologue<MODE, LAT_SMEM>(a, smem, lat_off, cpb, lane, wS, histS, gl);
    __syncthreads();
    ChainSetup<MODE, R> cs;
    cs.init(a, cpb, lane);
    const bool store = lane < cpb;
    int E = cs.active ? a.edel[cs.chain] : 0;
    int EJ = cs.active ? a.ej[cs.chain] : 0;
    int M = (cs.active && MODE == kModeProduce) ? a.mag[cs.chain] : 0;
    uint32_t c0 = 0;
    const uint32_t L = a.L, N = a.N, WPR = a.WPR;
    uint4 r1 = make_uint4(0, 0, 0, 0), r3 = r1;
    auto word_of = [&](uint32_t site) -> uint32_t * {
        const uint32_t r = site / L, c = site - r * L;
        return lat + (size_t)(r * WPR + (c >> 4)) * cpb;
    };
    auto get = [&](uint32_t site) -> int {
        const uint32_t c = site % L;
        return (int)spin_code(*word_of(site), c) - 1;
    };
    auto put = [&](uint32_t site, int s) {
        if (!store) return;
        const uint32_t c = site % L;
        uint32_t *p = word_of(site);
        const uint32_t sh = 2u * (c & 15u);
        *p = (*p & ~(3u << sh)) | ((uint32_t)(s + 1) << sh);
    };
    for (int phase = 0; phase < 2; ++phase) {
        const unsigned long long n = phase ? nup : a.therm;
        for (unsigned long long i = 0; i < n; ++i) {
            if ((i & 3ull) == 0) {
                ++c0;
                r1 = philox<R>(c0, cs.seed, iter, kCtrTag, cs.k1);
                r3 = philox<R>(c0, cs.seed, iter, kCtrTag, cs.k3);
            }
            const int sub = (int)(i & 3ull);
            const uint32_t idx = a.index[i % N];
            int ns = get(idx) + 2 * (u01f(pick(r3, sub)) < 0.5f) - 1;
            const int os = get(idx);
            ns = ns - 3 * (ns == 2) + 3 * (ns == -2);
            // the reference stores the trial value new*(old==0)+old before forming dE
            const int tmp = ns * (os == 0) + os;
            const int dE = ((os == 0) + os * (ns - os)) * (-tmp) *
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
            }
            if (phase == 1 && cs.active) record<MODE>(histS, a.hist, E, M);
        }
    }
    if (LAT_SMEM && store) {
        const uint32_t words = L * WPR;
        for (uint32_t w = 0; w < words; ++w) gl[(size_t)w * cpb] = lat[(size_t)w * cpb];
    }
    if (cs.active) {
        a.edel[cs.chain] = E;
        a.ej[cs.chain] = EJ;
        if (MODE == kModeProduce) a.mag[cs.chain] = M;
    }
    __syncthreads();
    drain_hist<MODE>(histS, a.hist, N);
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

// ---------------------------------------------------------------------------
SweepPlan plan_sweep(int mode, int rounds, uint32_t L, uint32_t nchains, size_t smem_optin, int sms, int kernel)
{
    SweepPlan p{};
    p.mode = mode;
    p.rounds = rounds;
    p.fast = (L % 8 == 0) && L >= 8;
    p.kernel = !p.fast ? kKernelGeneric : (kernel < 0 ? kKernelWindowed : kernel);
    const uint32_t N = L * L, WPR = (L + 15) / 16;
    const size_t per_chain = (size_t)L * WPR * 4;
    // chains per SM if spread over all SMs, rounded up to a warp, at most 128
    const uint32_t per_sm = (nchains + (uint32_t)sms - 1) / (uint32_t)sms;
    const uint32_t want = std::min<uint32_t>(128u, (per_sm + 31u) / 32u * 32u);
    const size_t base = smem_weights_bytes(mode, N) + smem_hist_bytes(mode, N);
    const size_t fixed = base + (p.kernel == kKernelSpecialized ? smem_ring_bytes((want + 31u) / 32u) : 0);
    const size_t cap = smem_optin > fixed ? (smem_optin - fixed) / per_chain : 0;
    uint32_t cpb = want;
    // Lattice in shared memory when a block of at least one warp fits and that
    // takes no more waves of blocks than keeping it in global memory (one
    // block of `want` chains per SM, served by L1/L2) would.
    p.lat_smem = false;
    if (cap >= 32) {
        uint32_t c = (uint32_t)std::min<size_t>(cap, want);
        if (p.kernel == kKernelGeneric) c = c / 32u * 32u;  // whole warps, no padding lanes there
        const uint32_t blocks = (nchains + c - 1) / c;
        if (p.kernel != kKernelGeneric) c = (nchains + blocks - 1) / blocks;  // evened out over the blocks
        const uint32_t waves_smem = (blocks + (uint32_t)sms - 1) / (uint32_t)sms;
        const uint32_t blocks_g = (nchains + want - 1) / want;
        const uint32_t waves_glob = (blocks_g + (uint32_t)sms - 1) / (uint32_t)sms;
        if (waves_smem <= waves_glob) {
            p.lat_smem = true;
            cpb = c;
        }
    }
    p.cpb = cpb;
    p.blocks = (nchains + cpb - 1) / cpb;
    const uint32_t warps = (cpb + 31u) / 32u;
    p.threads = (p.kernel == kKernelSpecialized ? 2u : 1u) * warps * 32u;
    p.smem = base + (p.kernel == kKernelSpecialized ? smem_ring_bytes(warps) : 0) +
             (p.lat_smem ? per_chain * cpb : 0);
    return p;
}

template <int MODE, int R, bool LS>
static cudaError_t launch_one(const SweepPlan &p, const SweepArgs &a, cudaStream_t s)
{
    void (*kern)(const SweepArgs, uint32_t) = p.kernel == kKernelSpecialized ? k_sweep_spec<MODE, R, LS>
                                            : p.kernel == kKernelWindowed    ? k_sweep_win<MODE, R, LS>
                                                                             : k_sweep_generic<MODE, R, LS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem);
    if (e != cudaSuccess) return e;
    kern<<<p.blocks, p.threads, p.smem, s>>>(a, p.cpb);
    return cudaGetLastError();
}

cudaError_t launch_sweep(const SweepPlan &p, const SweepArgs &a, cudaStream_t s)
{
    // the generic kernel reads the sweep order and neighbours from tables
    if (p.kernel == kKernelGeneric && (a.index == nullptr || a.naver == nullptr)) return cudaErrorInvalidValue;
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
