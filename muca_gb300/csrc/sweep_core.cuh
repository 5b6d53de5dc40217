// sweep_core.cuh -- the per-chain Metropolis machinery shared by the sweep
// kernels of one simulation (k_sweep.cu) and of a batch of simulations
// (k_batch.cu): shared-memory layout, Philox draws, the windowed SWAR step,
// the step-by-step partial window, histogram recording and the walk over the
// reference's sweep order.  See k_sweep.cu for the design.
#pragma once
#include "muca_device.cuh"
#include "muca_internal.h"

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
// ring: [pair][depth][word 0..kSlotWords-1][lane 0..31] u32, then the
// full/empty mbarriers of every pair and slot
__host__ __device__ inline size_t smem_ring_bytes(uint32_t pairs)
{
    return (size_t)pairs * kRingDepth * kSlotWords * 32 * 4 + (size_t)pairs * kRingDepth * 2 * 8;
}

struct ChainState {
    int E, EJ, M;
};

// A packed random word per attempt (the step-by-step partial windows take
// these): bits 31..8 are the top 24 bits of the acceptance draw r1 (all that
// u01fixedpt<float> uses: u = (1|(r1>>8)) 2^-24), bit 0 is the direction bit
// (u01fixedpt<float>(r3) < 0.5 <=> r3 < 2^31, so the bit is r3's top bit,
// set for s -> s-1).
__device__ __forceinline__ uint32_t pack_draw(uint32_t r1, uint32_t r3) { return (r1 & 0xFFFFFF00u) | (r3 >> 31); }

// One Philox block of the acceptance stream (k1) and one of the direction
// stream (k3) at the same counter (muca_delta_multigpu.cu:794-797), kept
// apart: r1[] the acceptance words (u01fixedpt uses their bits 31..9 only,
// as it does those of a packed word), r3[] the direction words (bit 31).
template <int R>
__device__ __forceinline__ void draw_pair(uint32_t cc, uint32_t seed, uint32_t iter, const RoundKeys<R> &k1,
                                          const RoundKeys<R> &k3, uint32_t *r1, uint32_t *r3)
{
    const uint4 a = philox<R>(cc, seed, iter, kCtrTag, k1);
    const uint4 b = philox<R>(cc, seed, iter, kCtrTag, k3);
    r1[0] = a.x; r1[1] = a.y; r1[2] = a.z; r1[3] = a.w;
    r3[0] = b.x; r3[1] = b.y; r3[2] = b.z; r3[3] = b.w;
}


// Histogram entry.  The u32 shared bins are drained into the u64 device
// histogram by the lane whose increment finds 2^31 counts already there.
template <int MODE, bool HS = true>
__device__ __forceinline__ void record(uint32_t *histS, unsigned long long *histG, int E, int M)
{
    if (MODE == kModeWeight && !HS) {
        atomicAdd(&histG[E], 1ull);
    } else if (MODE == kModeWeight) {
        const uint32_t old = atomicAdd(&histS[E], 1u);
        if (old >= 0x80000000u) {
            const uint32_t v = atomicExch(&histS[E], 0u);
            atomicAdd(&histG[E], (unsigned long long)v);
        }
    } else {
        atomicAdd(&histG[(uint32_t)(M + E * E + 2 * E) >> 1], 1ull);
    }
}

// Histogram entries of one window.  Weight mode with the shared u32
// histogram: one shared atomic per attempt; `checked` (uniform: the launch
// can put 2^32 entries into one block's bins) drains a u32 shared bin into
// the u64 device histogram once it holds 2^31 (the warp-specialised sweep;
// the windowed sweep flushes all bins between rows instead, flush_hist).
// Device (u64) histograms: the entries are merged into runs of equal bins
// per lane first (E_Delta moves by at most one per attempt, so a window's
// entries cluster), which saves global atomics; HS = false (weight mode)
// sends the runs straight to the u64 device histogram.
template <int MODE, int SLOTS, bool HS = true>
__device__ __forceinline__ void record_window(uint32_t *__restrict__ histS, unsigned long long *__restrict__ histG,
                                              const int (&Es)[SLOTS], const int (&Ms)[SLOTS], bool checked)
{
    // run lengths are at most SLOTS: 32-bit counts, widened at the atomics
    if (MODE == kModeWeight && !HS) {
        int cur = Es[0];
        uint32_t cnt = 1;
#pragma unroll
        for (int t = 1; t < SLOTS; ++t) {
            const bool same = Es[t] == cur;
            if (!same) atomicAdd(&histG[cur], (unsigned long long)cnt);
            cnt = same ? cnt + 1u : 1u;
            cur = Es[t];
        }
        atomicAdd(&histG[cur], (unsigned long long)cnt);
    } else if (MODE == kModeWeight) {
        if (checked) {
#pragma unroll
            for (int t = 0; t < SLOTS; ++t) {
                const uint32_t old = atomicAdd(&histS[Es[t]], 1u);
                if (old >= 0x80000000u) atomicAdd(&histG[Es[t]], (unsigned long long)atomicExch(&histS[Es[t]], 0u));
            }
            return;
        }
        // one fire-and-forget shared atomic per attempt: cheaper in issue
        // slots than merging runs of equal bins first (measured)
#pragma unroll
        for (int t = 0; t < SLOTS; ++t) atomicAdd(&histS[Es[t]], 1u);
    } else {
        uint32_t cur = (uint32_t)(Ms[0] + Es[0] * Es[0] + 2 * Es[0]) >> 1;
        uint32_t cnt = 1;
#pragma unroll
        for (int t = 1; t < SLOTS; ++t) {
            const uint32_t b = (uint32_t)(Ms[t] + Es[t] * Es[t] + 2 * Es[t]) >> 1;
            const bool same = b == cur;
            if (!same) atomicAdd(&histG[cur], (unsigned long long)cnt);
            cnt = same ? cnt + 1u : 1u;
            cur = b;
        }
        atomicAdd(&histG[cur], (unsigned long long)cnt);
    }
}

// A decoded window: everything its accept/reject scan needs, formed from the
// lattice words and the draws before the scan runs.
template <int MODE>
struct WinDec {
    using WT = typename WeightType<MODE>::T;
    uint32_t *pc;               // the window's lattice word
    uint32_t C, ctr, vnib, hs0;  // the word, old and proposed codes (nibbles), parity shift
    int dE[8], dDel[8], dM[8];
    float f2[8];                // -beta dE (an even integer for beta = 2: exact in FP32 and FP64)
    float lf[8];                // __logf(u)
    uint32_t p[8];              // the acceptance words (for the exact replay; bits 31..9 used)
    const uint32_t *pr;         // or, when set, those words in shared memory (pr[32 t])
};

// Decodes the SLOTS same-parity sites (half 0: even, 1: odd) of word q of
// row `row`, SLOTS consecutive attempts of the sweep, with the acceptance
// words r1[] and direction words r3[] of draw_pair.
// lat points at this lane's word 0 (stride cpb).  The half is a value, not a
// template branch, so decode and scan of neighbouring windows form one basic
// block the compiler can interleave.
// BT: -beta*dE comes from the table btab[dE + 8] (any beta) instead of the
// reference's literal -2 dE (beta = 2); the table holds (float)(-beta*dE),
// which for beta = 2 is the same value.
// rmask: rows are addressed as (row & rmask): ~0u for a whole lattice,
// 3 for the four-row ring of RowRing (L is a multiple of 4, so the ring's
// slots follow the periodic rows).
template <int MODE, int SLOTS, bool BT = false>
__device__ __forceinline__ void decode_window(uint32_t *__restrict__ lat, uint32_t cpb, uint32_t L, uint32_t WPR,
                                              uint32_t row, uint32_t q, uint32_t half, const uint32_t *r1,
                                              const uint32_t *r3, const float *__restrict__ btab, WinDec<MODE> &d,
                                              uint32_t rmask = ~0u)
{
    using WT = typename WeightType<MODE>::T;
    constexpr uint32_t M2 = 0x33333333u, N1 = 0x11111111u;
    const uint32_t rup = (row + 1 == L) ? 0u : row + 1;
    const uint32_t rdn = (row == 0) ? L - 1 : row - 1;
    const uint32_t rw = row & rmask;
    d.pc = lat + (size_t)(rw * WPR + q) * cpb;
    const uint32_t C = *d.pc;
    const uint32_t U = lat[(size_t)((rup & rmask) * WPR + q) * cpb];
    const uint32_t D = lat[(size_t)((rdn & rmask) * WPR + q) * cpb];
    // the one neighbour outside word q: left of the first even site, or
    // right of the last odd site (wrapping along the row)
    const uint32_t sq = half ? ((16 * q + 16 < L) ? q + 1 : 0u) : (q ? q - 1 : (L - 1) >> 4);
    const uint32_t sb = half ? 0u : (q ? 15u : ((L - 1) & 15u));
    const uint32_t sv = spin_code(lat[(size_t)(rw * WPR + sq) * cpb], sb);

    // Nibble t of `ctr` holds the spin code (s+1) of the window's site t;
    // nibble t of `nbs` the sum of its four neighbours' codes (0..8, no
    // carries).  `oth` holds the other parity's codes: for even sites the
    // right neighbours (shifted up: the left ones, with sv entering at t=0),
    // for odd sites the left neighbours (shifted down: the right ones, sv at
    // the top).
    const uint32_t hs0 = half ? 2u : 0u;
    const uint32_t ctr = (C >> hs0) & M2;
    const uint32_t oth = (C >> (2u - hs0)) & M2;
    const uint32_t side = half ? ((oth >> 4) | (sv << (4 * (SLOTS - 1)))) : ((oth << 4) | sv);
    const uint32_t nbs = oth + side + ((U >> hs0) & M2) + ((D >> hs0) & M2);
    // Proposals of all sites at once, nibble-parallel:  s -> s +/- 1 with the
    // cyclic wrap is code -> (code + 1 + d) mod 3, d the direction bit.
    uint32_t dn = 0;
#pragma unroll
    for (int t = 0; t < SLOTS; ++t) dn |= (r3[t] >> 31) << (4 * t);
    const uint32_t x = ctr + N1 + dn;                              // 1..4
    const uint32_t ge3 = ((x + N1) >> 2) & N1;                     // 1 where x >= 3
    const uint32_t vnib = x - (ge3 + (ge3 << 1));                  // new codes 0..2
    const uint32_t nzo = ((ctr ^ N1) | ((ctr ^ N1) >> 1)) & N1;    // s_old != 0
    const uint32_t nzn = ((vnib ^ N1) | ((vnib ^ N1) >> 1)) & N1;  // s_new != 0
    const uint32_t ddb = nzn + N1 - nzo;                           // dDel + 1 (0..2)
    const uint32_t dvb = vnib + 0x22222222u - ctr;                 // s_new - s_old + 2 (0..4)
    d.pr = nullptr;
    d.C = C;
    d.ctr = ctr;
    d.vnib = vnib;
    d.hs0 = hs0;
#pragma unroll
    for (int t = 0; t < SLOTS; ++t) {
        const int dv = (int)((dvb >> (4 * t)) & 7u) - 2;
        d.dDel[t] = (int)((ddb >> (4 * t)) & 3u) - 1;
        d.dE[t] = dv * (4 - (int)((nbs >> (4 * t)) & 15u));  // -(s_new - s_old) * (sum of neighbour spins)
        d.dM[t] = dv;
        if (BT) d.f2[t] = btab[d.dE[t] + 8];
        else    d.f2[t] = small_int_to_float(-2 * d.dE[t]);
        d.lf[t] = __logf(u01f(r1[t]));
        d.p[t] = r1[t];
    }
}

// The accept/reject scan of a decoded window, its lattice write and its
// histogram entries.  ONEBAND (weight mode): decide each attempt with the
// one-band test of the production scan instead of the two tests.  AHEAD2
// (weight mode): fetch each attempt's weight three attempts ahead, for the
// four outcomes of the two decisions between, instead of one attempt ahead
// for two outcomes.  Both forms decide every attempt identically; which is
// faster depends on the kernel around the scan (measured per kernel).
// `store` is false for padding lanes: they read another lane's spins, never
// accept (so their E stays at 3 and every weight index E + dDel_t + dDel_t+1
// + dDel_t+2 stays in [0, 6]) and never write.
template <int MODE, int SLOTS, bool HS = true, bool ONEBAND = false, bool AHEAD2 = false>
__device__ __forceinline__ void scan_window(const WinDec<MODE> &d, bool rec, bool store, bool checked,
                                            const typename WeightType<MODE>::T *__restrict__ wS,
                                            uint32_t *__restrict__ histS, unsigned long long *__restrict__ histG,
                                            ChainState &st, typename WeightType<MODE>::T eps,
                                            const double *__restrict__ wG = nullptr, float tol = 0.0f)
{
    using WT = typename WeightType<MODE>::T;
    constexpr uint32_t M2 = 0x33333333u;
    if (MODE == kModeProduce) {
        // Production: the reference forms diff in FP64 (produce2_multigpu.cu:474),
        // and FP64 issues slowly on this GPU.  The scan runs in FP32 on the
        // staged differences T[E] (prologue<..., DT>): fast = f2 + T[E].dDel,
        // within `tol` of the FP64 diff.  Any lane where that leaves the
        // decision in doubt sends the warp to the exact FP64 replay of the
        // window, with the FP64 weights in global memory, so every decision
        // is the reference's.
        const float2 *T = reinterpret_cast<const float2 *>(wS);
        const ChainState s0 = st;
        const float band = tol + (float)eps;
        float2 tE = T[st.E];
        float2 tN = T[st.E + d.dDel[0]];
        uint32_t accm = 0;
        bool near = false;
        int Es[SLOTS], Ms[SLOTS];
#pragma unroll
        for (int t = 0; t < SLOTS; ++t) {
            const int dd = d.dDel[t];
            const float dl = dd == 0 ? 0.0f : (dd < 0 ? tE.x : tE.y);
            const float fast = __fadd_rn(d.f2[t], dl);
            // logf(u) < 0 for every u = (1|(r>>8)) 2^-24 <= 1 - 2^-24, so the
            // reference's  diff >= 0 || logf(u) < diff  is  logf(u) < diff.
            // With |fast - diff| <= tol (any dDel, a zero difference
            // included) and |__logf(u) - logf(u)| <= eps, the sign of
            // g = __logf(u) - fast is that of logf(u) - diff whenever
            // |g| > tol + eps; otherwise the window is replayed.
            const float g = __fsub_rn(d.lf[t], fast);
            const bool acc = store && (g < 0.0f);
            near |= fabsf(g) <= band;
            if (acc) {
                st.E += dd;
                st.EJ += d.dE[t];
                st.M += d.dM[t];
                tE = tN;
                accm |= 0xFu << (4 * t);
            }
            Es[t] = st.E;
            Ms[t] = st.M;
            if (t + 1 < SLOTS) tN = T[st.E + d.dDel[t + 1]];
        }
        if (__any_sync(0xffffffffu, near)) {
            st = s0;
            accm = 0;
#pragma unroll
            for (int t = 0; t < SLOTS; ++t) {
                const double diff = __dsub_rn(__dadd_rn((double)d.f2[t], wG[st.E + d.dDel[t]]), wG[st.E]);
                bool acc = diff >= 0.0;
                if (!acc) acc = (double)logf(u01f(d.pr ? d.pr[32 * t] : d.p[t])) < diff;
                acc = acc && store;
                if (acc) {
                    st.E += d.dDel[t];
                    st.EJ += d.dE[t];
                    st.M += d.dM[t];
                    accm |= 0xFu << (4 * t);
                }
                Es[t] = st.E;
                Ms[t] = st.M;
            }
        }
        const uint32_t merged = (d.ctr & ~accm) | (d.vnib & accm);
        if (store) *d.pc = (d.C & (d.hs0 ? M2 : ~M2)) | (merged << d.hs0);
        if (rec) record_window<MODE, SLOTS, HS>(histS, histG, Es, Ms, checked);
        return;
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
    uint32_t accm = 0;
    bool near = false;
    int Es[SLOTS], Ms[SLOTS];
    if constexpr (AHEAD2) {
        // P[u][2a + b]: the weight at attempt u's proposed E_Delta when the
        // attempts u-2 and u-1 decide a and b, loaded after attempt u-3
        WT P[SLOTS][4];
        bool av[SLOTS];
        P[0][0] = wS[st.E + d.dDel[0]];
        if (SLOTS > 1) {
            P[1][0] = wS[st.E + d.dDel[1]];
            P[1][1] = wS[st.E + d.dDel[0] + d.dDel[1]];
        }
        if (SLOTS > 2) {
            P[2][0] = wS[st.E + d.dDel[2]];
            P[2][1] = wS[st.E + d.dDel[1] + d.dDel[2]];
            P[2][2] = wS[st.E + d.dDel[0] + d.dDel[2]];
            P[2][3] = wS[st.E + d.dDel[0] + d.dDel[1] + d.dDel[2]];
        }
#pragma unroll
        for (int t = 0; t < SLOTS; ++t) {
            WT A;
            if (t == 0) {
                A = P[0][0];
            } else if (t == 1) {
                A = av[0] ? P[1][1] : P[1][0];
            } else {
                const WT q0 = av[t - 2] ? P[t][2] : P[t][0];
                const WT q1 = av[t - 2] ? P[t][3] : P[t][1];
                A = av[t - 1] ? q1 : q0;
            }
            WT diff;
            if (MODE == kModeWeight)
                diff = __fsub_rn(__fadd_rn((float)d.f2[t], (float)A), (float)wE);
            else
                diff = __dsub_rn(__dadd_rn((double)d.f2[t], (double)A), (double)wE);
            const WT l = (WT)d.lf[t];
            bool acc;
            if (ONEBAND) {
                const WT g = l - diff;
                acc = store && (g < (WT)0);
                near |= fabs(g) <= eps;
            } else {
                acc = store && ((diff >= (WT)0) || (l < diff));
                near |= (diff < (WT)0) && (fabs(l - diff) <= eps);
            }
            av[t] = acc;
            if (acc) {
                st.E += d.dDel[t];
                st.EJ += d.dE[t];
                st.M += d.dM[t];
                wE = A;
                accm |= 0xFu << (4 * t);
            }
            Es[t] = st.E;
            Ms[t] = st.M;
            if (t + 3 < SLOTS) {
                const int e = st.E + d.dDel[t + 3];
                P[t + 3][0] = wS[e];
                P[t + 3][1] = wS[e + d.dDel[t + 2]];
                P[t + 3][2] = wS[e + d.dDel[t + 1]];
                P[t + 3][3] = wS[e + d.dDel[t + 1] + d.dDel[t + 2]];
            }
        }
    } else {
        WT A = wS[st.E + d.dDel[0]];
        WT c0 = A, c1 = A;
        if (SLOTS > 1) {
            c0 = wS[st.E + d.dDel[1]];
            c1 = wS[st.E + d.dDel[0] + d.dDel[1]];
        }
#pragma unroll
        for (int t = 0; t < SLOTS; ++t) {
            WT diff;
            if (MODE == kModeWeight)
                diff = __fsub_rn(__fadd_rn((float)d.f2[t], (float)A), (float)wE);
            else
                diff = __dsub_rn(__dadd_rn((double)d.f2[t], (double)A), (double)wE);
            const WT l = (WT)d.lf[t];
            bool acc;
            if (ONEBAND) {
                // logf(u) < 0 for every u <= 1 - 2^-24, so  diff >= 0 || logf(u) < diff
                // is  logf(u) < diff;  g = __logf(u) - diff has its sign unless |g| <= eps
                const WT g = l - diff;
                acc = store && (g < (WT)0);
                near |= fabs(g) <= eps;
            } else {
                // two tests: the one-band form measured 11 % slower in the
                // single-instance kernel (and 1 % faster in the batch kernel)
                acc = store && ((diff >= (WT)0) || (l < diff));
                near |= (diff < (WT)0) && (fabs(l - diff) <= eps);
            }
            if (acc) {
                st.E += d.dDel[t];
                st.EJ += d.dE[t];
                st.M += d.dM[t];
                wE = A;
                accm |= 0xFu << (4 * t);
            }
            Es[t] = st.E;
            Ms[t] = st.M;
            if (t + 1 < SLOTS) {
                A = acc ? c1 : c0;
                if (t + 2 < SLOTS) {
                    c0 = wS[st.E + d.dDel[t + 2]];
                    c1 = wS[st.E + d.dDel[t + 1] + d.dDel[t + 2]];
                }
            }
        }
    }
    if (__any_sync(0xffffffffu, near)) {
        st = s0;
        wE = wE0;
        accm = 0;
#pragma unroll
        for (int t = 0; t < SLOTS; ++t) {
            const WT wn = wS[st.E + d.dDel[t]];
            WT diff;
            if (MODE == kModeWeight)
                diff = __fsub_rn(__fadd_rn((float)d.f2[t], (float)wn), (float)wE);
            else
                diff = __dsub_rn(__dadd_rn((double)d.f2[t], (double)wn), (double)wE);
            bool acc = diff >= (WT)0;
            if (!acc) acc = (WT)logf(u01f(d.pr ? d.pr[32 * t] : d.p[t])) < diff;
            acc = acc && store;
            if (acc) {
                st.E += d.dDel[t];
                st.EJ += d.dE[t];
                st.M += d.dM[t];
                wE = wn;
                accm |= 0xFu << (4 * t);
            }
            Es[t] = st.E;
            Ms[t] = st.M;
        }
    }
    const uint32_t merged = (d.ctr & ~accm) | (d.vnib & accm);
    if (store) *d.pc = (d.C & (d.hs0 ? M2 : ~M2)) | (merged << d.hs0);
    if (rec) record_window<MODE, SLOTS, HS>(histS, histG, Es, Ms, checked);
}

// One full window: decode, then scan.
template <int MODE, int SLOTS, int HALF, bool HS = true, bool BT = false, bool AHEAD2 = false>
__device__ __forceinline__ void window_core(uint32_t *__restrict__ lat, uint32_t cpb, uint32_t L, uint32_t WPR,
                                            uint32_t row, uint32_t q, bool rec, bool store, bool checked,
                                            const typename WeightType<MODE>::T *__restrict__ wS,
                                            uint32_t *__restrict__ histS, unsigned long long *__restrict__ histG,
                                            ChainState &st, const uint32_t (&r1)[SLOTS], const uint32_t (&r3)[SLOTS],
                                            typename WeightType<MODE>::T eps, const float *__restrict__ btab = nullptr,
                                            uint32_t hrt = 0, const double *__restrict__ wG = nullptr,
                                            float tol = 0.0f, uint32_t rmask = ~0u)
{
    WinDec<MODE> d;
    decode_window<MODE, SLOTS, BT>(lat, cpb, L, WPR, row, q, HALF < 0 ? hrt : (uint32_t)HALF, r1, r3, btab, d,
                                   rmask);
    // the batch kernel (the one user of the beta table) and the scan with
    // weights fetched three attempts ahead decide weight-mode attempts with
    // the one-band test
    scan_window<MODE, SLOTS, HS, BT || AHEAD2, AHEAD2>(d, rec, store, checked, wS, histS, histG, st, eps, wG, tol);
}

// The first `len` (< window size) attempts of a window, one at a time as
// the reference writes them; only the last window of a phase is partial.
template <int MODE, bool HS = true, bool BT = false>
__device__ __noinline__ void partial_core(uint32_t *__restrict__ lat, uint32_t cpb, uint32_t L, uint32_t WPR,
                                          uint32_t row, uint32_t q, uint32_t half, uint32_t len, bool rec,
                                          bool store, const typename WeightType<MODE>::T *__restrict__ wS,
                                          uint32_t *__restrict__ histS, unsigned long long *__restrict__ histG,
                                          ChainState &st, const uint32_t *p, const float *__restrict__ btab = nullptr,
                                          uint32_t rmask = ~0u)
{
    using WT = typename WeightType<MODE>::T;
    const uint32_t rup = ((row + 1 == L) ? 0u : row + 1) & rmask;
    const uint32_t rdn = ((row == 0) ? L - 1 : row - 1) & rmask;
    const uint32_t rw = row & rmask;
    for (uint32_t t = 0; t < len; ++t) {
        const uint32_t col = 16u * q + 2u * t + half;
        const uint32_t cl = col ? col - 1 : L - 1, cr = (col + 1 == L) ? 0u : col + 1;
        uint32_t *pw = lat + (size_t)(rw * WPR + (col >> 4)) * cpb;
        const int os = (int)spin_code(*pw, col) - 1;
        int ns = os + ((p[t] & 1u) ? -1 : 1);
        ns = ns - 3 * (ns == 2) + 3 * (ns == -2);
        const int nb = (int)spin_code(lat[(size_t)(rw * WPR + (cl >> 4)) * cpb], cl) +
                       (int)spin_code(lat[(size_t)(rw * WPR + (cr >> 4)) * cpb], cr) +
                       (int)spin_code(lat[(size_t)(rup * WPR + (col >> 4)) * cpb], col) +
                       (int)spin_code(lat[(size_t)(rdn * WPR + (col >> 4)) * cpb], col) - 4;
        const int dE = -(ns - os) * nb, dDel = ns * ns - os * os, dM = ns - os;
        const WT f2 = BT ? (WT)btab[dE + 8] : (WT)(-2 * dE);
        WT diff;
        if (MODE == kModeWeight)
            diff = __fsub_rn(__fadd_rn((float)f2, (float)wS[st.E + dDel]), (float)wS[st.E]);
        else
            diff = __dsub_rn(__dadd_rn((double)f2, (double)wS[st.E + dDel]), (double)wS[st.E]);
        bool acc = diff >= (WT)0;
        if (!acc) acc = (WT)logf(u01f(p[t])) < diff;
        if (acc && store) {
            const uint32_t sh = 2u * (col & 15u);
            *pw = (*pw & ~(3u << sh)) | ((uint32_t)(ns + 1) << sh);
            st.E += dDel;
            st.EJ += dE;
            st.M += dM;
        }
        if (rec) record<MODE, HS>(histS, histG, st.E, st.M);
    }
}

// Stages the FP32 differences T[E] = {w[E-1] - w[E], w[E+1] - w[E]} of the
// FP64 weights w[0..N] in shared memory (every thread of the block calls it)
// and returns the bound `tol` of the FP32 fast difference
// fast = f2 + T[E].(dDel) against the reference's FP64
// diff = ((double)f2 + w[E + dDel]) - w[E], |f2| <= 16:
//   |fast - diff| <= 2^-24 (|T| + |fast|) + 2^-53 (|w| + 16 + |diff| + |T|),
// with |T| and |w| reduced over the block, |fast|, |diff| <= 16 + max|T|;
// twice that.
__device__ __forceinline__ float stage_diff_table(const double *__restrict__ w64, uint32_t N, float2 *T)
{
    __shared__ float s_md[32];
    __shared__ double s_mw[32];
    const uint32_t nt = blockDim.x, tid = threadIdx.x;
    float md = 0.0f;
    double mw = 0.0;
    for (uint32_t i = tid; i <= N; i += nt) {
        const double w0 = w64[i];
        const float dm = i > 0 ? (float)__dsub_rn(w64[i - 1], w0) : 0.0f;
        const float dp = i < N ? (float)__dsub_rn(w64[i + 1], w0) : 0.0f;
        T[i] = make_float2(dm, dp);
        md = fmaxf(md, fmaxf(fabsf(dm), fabsf(dp)));
        mw = fmax(mw, fabs(w0));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        md = fmaxf(md, __shfl_xor_sync(0xffffffffu, md, o));
        mw = fmax(mw, __shfl_xor_sync(0xffffffffu, mw, o));
    }
    if ((tid & 31u) == 0) { s_md[tid >> 5] = md; s_mw[tid >> 5] = mw; }
    __syncthreads();
    if (tid == 0) {
        for (uint32_t k = 1; k < (nt + 31) / 32; ++k) { md = fmaxf(md, s_md[k]); mw = fmax(mw, s_mw[k]); }
        const double m = (double)md * 1.0001;
        s_md[0] = (float)((2.0 * 5.9604644775390625e-8 * (2.0 * m + 16.0) +
                           2.0 * 1.1102230246251565e-16 * (mw + 32.0 + 2.0 * m)) * 1.0001);
    }
    __syncthreads();
    const float tol = s_md[0];
    __syncthreads();
    return tol;
}

// Stage weights, clear the histogram, stage this block's lattice; returns
// the lane's lattice base (shared or global).  Only lanes < cpb copy.
// `blk` is the chain block (blockIdx.x for a single simulation).
// DT (production): instead of the FP64 weights, shared memory holds the
// FP32 differences T[E] = {w[E-1] - w[E], w[E+1] - w[E]} of the FP64 weights
// (same size), and *tol gets the bound of the FP32 fast test (see
// scan_window); the FP64 weights stay in global memory for the exact test.
template <int MODE, bool LAT_SMEM, bool HS = true, bool DT = false>
__device__ __forceinline__ uint32_t *prologue(const SweepArgs &a, unsigned char *smem, size_t lat_offset,
                                              uint32_t cpb, uint32_t lane, uint32_t blk,
                                              typename WeightType<MODE>::T *&wS, uint32_t *&histS, uint32_t *&gl,
                                              float *tol = nullptr)
{
    using WT = typename WeightType<MODE>::T;
    const uint32_t N = a.N, nt = blockDim.x, tid = threadIdx.x;
    wS = reinterpret_cast<WT *>(smem);
    histS = reinterpret_cast<uint32_t *>(smem + smem_weights_bytes(MODE, N));
    uint32_t *latS = reinterpret_cast<uint32_t *>(smem + lat_offset);
    const WT *wg = reinterpret_cast<const WT *>(a.w);
    if (MODE == kModeProduce && DT) {
        const float t = stage_diff_table(reinterpret_cast<const double *>(a.w), N,
                                         reinterpret_cast<float2 *>(smem));
        if (tol) *tol = t;
    } else {
        for (uint32_t i = tid; i <= N; i += nt) wS[i] = wg[i];
    }
    if (MODE == kModeWeight && HS)
        for (uint32_t i = tid; i <= N; i += nt) histS[i] = 0u;
    const uint32_t words = a.L * a.WPR;
    const uint32_t l = lane < cpb ? lane : 0u;  // padding lanes read lane 0's words, never write
    gl = a.lat + (size_t)blk * words * cpb + l;
    if (LAT_SMEM) {
        if (lane < cpb)
            for (uint32_t w = 0; w < words; ++w) latS[(size_t)w * cpb + lane] = gl[(size_t)w * cpb];
        return latS + l;
    }
    return gl;
}

// Four-row ring of one chain's lattice in shared memory, for lattices that
// stay in global memory.  A window of row r reads rows r - 1, r and r + 1
// (periodic) and writes row r, so only those rows need to be near: slot
// s = row & 3 of the ring holds row tag(s) (L is a multiple of 4, so the
// slots follow the periodic rows).  At the start of every row the ring makes
// rows r - 1 .. r + 1 resident (normally they already are) and starts
// loading row r + 2 from global memory into registers, after writing the
// slot's previous row (r - 2) back; those registers go into the slot at the
// start of the next row, so the global latency hides behind a whole row of
// windows.  A row that is not in its slot is not in the ring at all, so its
// global copy is current: jumps (a new phase restarts the sweep at row 0)
// fall back to loads at the row start.  Only the lane that owns the column
// (`store`) moves data; padding lanes read lane 0's ring and never write.
// WMAX >= words per row (8 for L <= 128).
template <int WMAX>
struct RowRing {
    uint32_t *rs;  // the lane's ring column: word (slot, q) at rs[(slot * WPR + q) * cpb]
    uint32_t *gs;  // the lane's global column: word (row, q) at gs[(row * WPR + q) * cpb]
    int t0, t1, t2, t3;  // row held by each slot, -1 for none
    int prow;            // row whose words wait in pw, -1 for none
    uint32_t pw[WMAX];

    __device__ __forceinline__ void init(uint32_t *ring_col, uint32_t *glob_col)
    {
        rs = ring_col;
        gs = glob_col;
        t0 = t1 = t2 = t3 = -1;
        prow = -1;
    }
    __device__ __forceinline__ int tag(int s) const { return s == 0 ? t0 : s == 1 ? t1 : s == 2 ? t2 : t3; }
    __device__ __forceinline__ void set_tag(int s, int v)
    {
        t0 = s == 0 ? v : t0;
        t1 = s == 1 ? v : t1;
        t2 = s == 2 ? v : t2;
        t3 = s == 3 ? v : t3;
    }
    __device__ __forceinline__ void writeback(int s, uint32_t cpb, uint32_t WPR, bool store)
    {
        const int r = tag(s);
        if (r < 0) return;
        if (store)
            for (uint32_t q = 0; q < WPR; ++q) gs[((size_t)r * WPR + q) * cpb] = rs[((size_t)s * WPR + q) * cpb];
        set_tag(s, -1);
    }
    __device__ __forceinline__ void load(int row, uint32_t cpb, uint32_t WPR, bool store)
    {
        const int s = row & 3;
        writeback(s, cpb, WPR, store);
        if (store)
            for (uint32_t q = 0; q < WPR; ++q) rs[((size_t)s * WPR + q) * cpb] = gs[((size_t)row * WPR + q) * cpb];
        set_tag(s, row);
    }
    __device__ __forceinline__ void row_start(uint32_t r, uint32_t L, uint32_t cpb, uint32_t WPR, bool store)
    {
        if (prow >= 0) {
            const int s = prow & 3;
            if (store) {
#pragma unroll
                for (int q = 0; q < WMAX; ++q)
                    if ((uint32_t)q < WPR) rs[((size_t)s * WPR + q) * cpb] = pw[q];
            }
            set_tag(s, prow);
            prow = -1;
        }
        const int rm = r == 0 ? (int)L - 1 : (int)r - 1, rc = (int)r, rp = r + 1 == L ? 0 : (int)r + 1;
        if (tag(rm & 3) != rm) load(rm, cpb, WPR, store);
        if (tag(rc & 3) != rc) load(rc, cpb, WPR, store);
        if (tag(rp & 3) != rp) load(rp, cpb, WPR, store);
        const int P = rp + 1 == (int)L ? 0 : rp + 1;
        const int s = P & 3;
        if (tag(s) != P) {
            writeback(s, cpb, WPR, store);
            if (store) {
#pragma unroll
                for (int q = 0; q < WMAX; ++q)
                    if ((uint32_t)q < WPR) pw[q] = gs[((size_t)P * WPR + q) * cpb];
            }
            prow = P;
        }
    }
    __device__ __forceinline__ void finish(uint32_t cpb, uint32_t WPR, bool store)
    {
        for (int s = 0; s < 4; ++s) writeback(s, cpb, WPR, store);
        prow = -1;
    }
};
__host__ __device__ inline size_t ring_bytes(uint32_t L, uint32_t cpb)
{
    return (size_t)4 * ((L + 15) / 16) * cpb * 4;
}

// Moves the shared u32 bins into the u64 device histogram and clears them;
// every thread of the block calls it (it holds two block barriers).
template <int MODE>
__device__ __forceinline__ void flush_hist(uint32_t *histS, unsigned long long *histG, uint32_t N)
{
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
    __device__ __forceinline__ void init(const SweepArgs &a, uint32_t cpb, uint32_t lane, uint32_t blk)
    {
        chain = blk * cpb + lane;
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


// The windowed sweep of chain block `blk` (cpb chains, lanes >= cpb are
// padding): every lane draws its own Philox numbers one window ahead (n1/n3
// hold the acceptance and direction words of the next two groups, counters
// cc-1, cc).  Ends
// with the block synchronised and, with HS, the shared histogram drained.
// RING (with LAT_SMEM false): the lattice stays in global memory and each
// lane keeps a four-row ring of its chain in shared memory (RowRing), at the
// offset where the whole lattice would go.
template <int MODE, int R, bool LAT_SMEM, bool HS = true, bool BT = false, bool RING = false, bool AHEAD2 = false>
__device__ __forceinline__ void win_sweep_block(const SweepArgs &a, unsigned char *smem, uint32_t cpb, uint32_t blk,
                                                uint32_t iter, unsigned long long nup,
                                                const float *__restrict__ btab = nullptr)
{
    static_assert(!(RING && LAT_SMEM), "the ring serves lattices in global memory");
    using WT = typename WeightType<MODE>::T;
    const uint32_t lane = threadIdx.x;
    WT *wS;
    uint32_t *histS, *gl;
    const size_t lat_off = smem_weights_bytes(MODE, a.N) + (HS ? smem_hist_bytes(MODE, a.N) : 0);
    constexpr bool DT = MODE == kModeProduce;  // production scans on the FP32 difference table
    float tol = 0.0f;
    uint32_t *lat = prologue<MODE, LAT_SMEM, HS, DT>(a, smem, lat_off, cpb, lane, blk, wS, histS, gl, &tol);
    RowRing<8> ring;
    if (RING) {
        ring.init(reinterpret_cast<uint32_t *>(smem + lat_off) + (lane < cpb ? lane : 0u), gl);
        lat = ring.rs;
    }
    constexpr uint32_t rmask = RING ? 3u : ~0u;
    __syncthreads();
    const double *wG = reinterpret_cast<const double *>(a.w);
    // the step-by-step path reads the weights it needs: FP64 ones from global memory in production
    const WT *wP = DT ? reinterpret_cast<const WT *>(a.w) : wS;
    ChainSetup<MODE, R> cs;
    cs.init(a, cpb, lane, blk);
    const bool store = lane < cpb;
    ChainState st;
    st.E = cs.active ? a.edel[cs.chain] : (store ? 0 : 3);
    st.EJ = cs.active ? a.ej[cs.chain] : 0;
    st.M = (cs.active && MODE == kModeProduce) ? a.mag[cs.chain] : 0;
    const WT eps = (WT)a.log_eps;
    const uint32_t L = a.L, WPR = a.WPR;
    // draws of the next two groups (counters cc - 1, cc), the two streams apart
    uint32_t n1[8], n3[8];
    draw_pair<R>(1u, cs.seed, iter, cs.k1, cs.k3, n1, n3);
    draw_pair<R>(2u, cs.seed, iter, cs.k1, cs.k3, n1 + 4, n3 + 4);
    uint32_t cc = 2;
    auto advance = [&](uint32_t groups) {
        if (groups == 2) {
            draw_pair<R>(cc + 1, cs.seed, iter, cs.k1, cs.k3, n1, n3);
            draw_pair<R>(cc + 2, cs.seed, iter, cs.k1, cs.k3, n1 + 4, n3 + 4);
            cc += 2;
        } else {
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                n1[t] = n1[t + 4];
                n3[t] = n3[t + 4];
            }
            draw_pair<R>(cc + 1, cs.seed, iter, cs.k1, cs.k3, n1 + 4, n3 + 4);
            cc += 1;
        }
    };
    // The reference's sweep order (for_each_window's): whole row-halves as a
    // loop of full windows, W8 words of 8 same-parity sites and, with
    // L % 16 == 8, one word of 4; a phase's last, partial row-half (only when
    // therm or nup is not a multiple of L/2) step by step.
    const uint32_t W8 = L >> 4, per_row = L >> 1;
    const bool tail4 = (L & 15u) != 0;
    // recorded attempts per lane since the shared u32 bins were last flushed:
    // no bin can reach 2^32 while cpb * since stays below it
    unsigned long long since = 0;
    for (int phase = 0; phase < 2; ++phase) {
        unsigned long long n = phase ? nup : a.therm;
        const bool rec = phase == 1 && cs.active;
        uint32_t row = 0, half = 0;
        while (n >= per_row) {
            if (RING) ring.row_start(row, L, cpb, WPR, store);
            if (HS && MODE == kModeWeight && phase == 1) {
                if ((since + per_row) * cpb > 0xFFFFFFFFull || (a.hooks & kHookFlushRows)) {  // uniform
                    flush_hist<MODE>(histS, a.hist, a.N);
                    since = 0;
                }
                since += per_row;
            }
            for (uint32_t q = 0; q < W8; ++q) {
                uint32_t r1[8], r3[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    r1[t] = n1[t];
                    r3[t] = n3[t];
                }
                advance(2);  // independent of the window below: overlaps its scan
                window_core<MODE, 8, -1, HS, BT, AHEAD2>(lat, cpb, L, WPR, row, q, rec, store, false, wS, histS,
                                                         a.hist, st, r1, r3, eps, btab, half, wG, tol, rmask);
            }
            if (tail4) {
                uint32_t r1[4], r3[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    r1[t] = n1[t];
                    r3[t] = n3[t];
                }
                advance(1);
                window_core<MODE, 4, -1, HS, BT, AHEAD2>(lat, cpb, L, WPR, row, W8, rec, store, false, wS, histS,
                                                         a.hist, st, r1, r3, eps, btab, half, wG, tol, rmask);
            }
            n -= per_row;
            if (++row == L) {
                row = 0;
                half ^= 1u;
            }
        }
        if (n) {
            if (RING) ring.row_start(row, L, cpb, WPR, store);
            for (uint32_t q = 0; n; ++q) {
                const uint32_t cnt = (min(16u * q + 16u, L) - 16u * q) >> 1;
                const uint32_t len = n < cnt ? (uint32_t)n : cnt;
                uint32_t p[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) p[t] = pack_draw(n1[t], n3[t]);
                partial_core<MODE, HS, BT>(lat, cpb, L, WPR, row, q, half, len, rec, store, wP, histS, a.hist, st, p,
                                           btab, rmask);
                advance((len + 3u) >> 2);
                n -= len;
            }
        }
    }
    if (LAT_SMEM && store) {
        const uint32_t words = L * WPR;
        for (uint32_t w = 0; w < words; ++w) gl[(size_t)w * cpb] = lat[(size_t)w * cpb];
    }
    if (RING) ring.finish(cpb, WPR, store);
    if (cs.active) {
        a.edel[cs.chain] = st.E;
        a.ej[cs.chain] = st.EJ;
        if (MODE == kModeProduce) a.mag[cs.chain] = st.M;
    }
    __syncthreads();
    if (HS) drain_hist<MODE>(histS, a.hist, a.N);
}


}  // namespace muca
