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
//                 Philox numbers and decodes each window into a 2-deep
//                 shared-memory ring guarded by mbarriers, and one consumer
//                 warp runs the scan, write-back and histogram; two
//                 independent instruction streams per 32 chains;
//   k_sweep_win   the same window core with the Philox numbers drawn by the
//                 chain's own lane, one window ahead;
//   k_sweep_generic  the reference step by step on the packed layout, any L.
#include "sweep_core.cuh"

#include <algorithm>
#include <cstring>
#include <mutex>

namespace muca {

// ---------------------------------------------------------------------------
// Windowed kernel: one block per chain block, blockDim = cpb rounded up to a warp.
// RING: the lattice stays in global memory behind a four-row ring per lane.
template <int MODE, int R, bool LAT_SMEM, bool RING = false>
__global__ void __launch_bounds__(256, 1) k_sweep_win(const SweepArgs a, uint32_t cpb)
{
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t iter;
    unsigned long long nup;
    if (!launch_params(a, iter, nup)) return;
    // with the lattice behind the row ring the scan fetches weights three
    // attempts ahead (measured faster there, slower with the lattice in
    // shared memory)
    win_sweep_block<MODE, R, LAT_SMEM, true, false, RING, RING>(a, smem, cpb, blockIdx.x, iter, nup);
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
// Bounded wait: gives up once the phase has not completed for `limit` SM
// clock cycles (measured from this wait's start, so a long launch that keeps
// making progress never gives up).  Every lane of the calling warp waits on
// the same barrier at the same point; the outcome is voted across the warp,
// so a warp never splits between giving up and going on (the scan's
// warp-wide votes need all 32 lanes).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long limit)
{
    bool done = mbar_try_wait(bar, parity);
    if (!done) {
        const long long t0 = clock64();
        while (!(done = mbar_try_wait(bar, parity)))
            if (clock64() - t0 > limit) break;
    }
    return __all_sync(0xffffffffu, done);
}

// Slot words (index f: shared u32 at slot[32 f], one column per lane).
enum SlotWord : uint32_t {
    kSlotC = 0,     // the window's lattice word as the producer read it
    kSlotV = 1,     // proposed codes (nibbles)
    kSlotDD = 2,    // dDelta + 1 (nibbles)
    kSlotDV = 3,    // s_new - s_old + 2 (nibbles; production only)
    kSlotDE = 4,    // dE as signed bytes, sites 0..3 and 4..7 (two words)
    kSlotF2 = 6,    // -beta dE as floats (8 words)
    kSlotLF = 14,   // __logf(u) (8 words)
    kSlotP = 22,    // acceptance words for the exact replay, or packed draws of a partial window (8 words)
};
static_assert(kSlotP + 8 == kSlotWords, "slot layout");

// The producer's half of a window: decode (as decode_window) and store the
// fields the consumer's scan needs into the slot.
template <int MODE, int SLOTS>
__device__ __forceinline__ void put_window(const WinDec<MODE> &d, uint32_t *slot)
{
    slot[32 * kSlotC] = d.C;
    slot[32 * kSlotV] = d.vnib;
    uint32_t dd = 0, dv = 0, e0 = 0, e1 = 0;
#pragma unroll
    for (int t = 0; t < SLOTS; ++t) {
        dd |= (uint32_t)(d.dDel[t] + 1) << (4 * t);
        dv |= (uint32_t)(d.dM[t] + 2) << (4 * t);
        if (t < 4) e0 |= ((uint32_t)d.dE[t] & 0xFFu) << (8 * t);
        else       e1 |= ((uint32_t)d.dE[t] & 0xFFu) << (8 * (t - 4));
        slot[32 * (kSlotF2 + t)] = __float_as_uint(d.f2[t]);
        slot[32 * (kSlotLF + t)] = __float_as_uint(d.lf[t]);
        slot[32 * (kSlotP + t)] = d.p[t];
    }
    slot[32 * kSlotDD] = dd;
    if (MODE == kModeProduce) slot[32 * kSlotDV] = dv;
    slot[32 * kSlotDE] = e0;
    if (SLOTS > 4) slot[32 * (kSlotDE + 1)] = e1;
}

// The consumer's half: the decoded window back from the slot.  The word the
// producer read is still the word in the lattice: this parity's bits of it
// change only at this window, the other parity's only in the other half.
template <int MODE, int SLOTS>
__device__ __forceinline__ void get_window(const uint32_t *slot, uint32_t *pc, uint32_t half, WinDec<MODE> &d)
{
    constexpr uint32_t M2 = 0x33333333u;
    d.pc = pc;
    d.C = slot[32 * kSlotC];
    d.hs0 = half ? 2u : 0u;
    d.ctr = (d.C >> d.hs0) & M2;
    d.vnib = slot[32 * kSlotV];
    const uint32_t dd = slot[32 * kSlotDD];
    const uint32_t dv = MODE == kModeProduce ? slot[32 * kSlotDV] : 0u;
    const uint32_t e0 = slot[32 * kSlotDE];
    const uint32_t e1 = SLOTS > 4 ? slot[32 * (kSlotDE + 1)] : 0u;
#pragma unroll
    for (int t = 0; t < SLOTS; ++t) {
        d.dDel[t] = (int)((dd >> (4 * t)) & 3u) - 1;
        d.dM[t] = MODE == kModeProduce ? (int)((dv >> (4 * t)) & 7u) - 2 : 0;
        d.dE[t] = (int)(signed char)(uint8_t)((t < 4 ? e0 : e1) >> (8 * (t & 3)));
        d.f2[t] = __uint_as_float(slot[32 * (kSlotF2 + t)]);
        d.lf[t] = __uint_as_float(slot[32 * (kSlotLF + t)]);
    }
    d.pr = slot + 32 * kSlotP;
}

// Per 32 chains one producer warp and one consumer warp.  The producer draws
// the Philox numbers and decodes each window (proposals, dE, dDelta,
// __logf(u)) into a ring slot; the consumer runs the scan, the lattice
// store and the histogram.  Decoding window (row, q) reads the same-parity
// word of row - 1, written by the consumer WPR windows earlier, so the ring
// is at most WPR deep; at the start of a half (and of a phase) the producer
// waits until every earlier window is written back, since the new half reads
// the other parity.  A slot is released after its window's store, so a
// released slot also means a written word.  Every wait is bounded.
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
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + ring_off + (size_t)P * kRingDepth * kSlotWords * 32 * 4);
    uint64_t *full = bars + (size_t)pair * kRingDepth * 2;
    uint64_t *empty = full + kRingDepth;
    uint32_t *myring = ring + (size_t)pair * kRingDepth * kSlotWords * 32 + l32;
    if (threadIdx.x == 0) {
        for (uint32_t i = 0; i < P * kRingDepth * 2; ++i) mbar_init(bars + i, 32);
    }
    WT *wS;
    uint32_t *histS, *gl;
    const size_t lat_off = ring_off + smem_ring_bytes(P);
    constexpr bool DT = MODE == kModeProduce;  // production scans on the FP32 difference table
    float tol = 0.0f;
    uint32_t *lat = prologue<MODE, LAT_SMEM, true, DT>(a, smem, lat_off, cpb, producer ? 0xFFFFFFFFu : lane,
                                                       blockIdx.x, wS, histS, gl, &tol);
    if (producer) {  // the pair's lattice columns (padding lanes read lane 0's)
        const uint32_t l = lane < cpb ? lane : 0u;
        lat = LAT_SMEM ? reinterpret_cast<uint32_t *>(smem + lat_off) + l
                       : a.lat + (size_t)blockIdx.x * a.L * a.WPR * cpb + l;
    }
    const double *wG = reinterpret_cast<const double *>(a.w);
    const WT *wP = DT ? reinterpret_cast<const WT *>(a.w) : wS;
    __syncthreads();
    ChainSetup<MODE, R> cs;
    cs.init(a, cpb, lane, blockIdx.x);
    const uint32_t L = a.L, WPR = a.WPR;
    // depth D: the largest power of two <= min(kRingDepth, WPR)
    uint32_t dsh = 0;
    while ((2u << dsh) <= kRingDepth && (2u << dsh) <= WPR) ++dsh;
    const uint32_t D = 1u << dsh;
    const long long limit = a.wait_cycles > 0 ? a.wait_cycles : kWaitCyclesDefault;
    const bool silent = (a.hooks & kHookSilentProducer) != 0;
    uint32_t w = 0;  // window counter (ring position)
    bool ok = true;

    if (producer) {
        uint32_t cc = 0;  // Philox counter word 0 of the last drawn group
        for_each_window(L, WPR, a.therm, nup, [&](uint32_t row, uint32_t q, uint32_t half, uint32_t cnt,
                                                  uint32_t len, bool) {
            uint32_t r1[8], r3[8];
            draw_pair<R>(cc + 1, cs.seed, iter, cs.k1, cs.k3, r1, r3);
            if (len > 4) draw_pair<R>(cc + 2, cs.seed, iter, cs.k1, cs.k3, r1 + 4, r3 + 4);
#pragma unroll
            for (int t = 0; t < 4; ++t)
                if (len <= 4) r1[4 + t] = r3[4 + t] = 0u;
            cc += (len + 3u) >> 2;
            if (row == 0 && q == 0) {
                // a new half or phase: the windows still in the ring must be written back
                for (uint32_t j = 1; j < D && j <= w; ++j) {
                    const uint32_t v = w - j;
                    if (!mbar_wait(empty + (v & (D - 1u)), (v >> dsh) & 1u, limit)) { ok = false; return false; }
                }
            }
            const uint32_t s = w & (D - 1u), round = w >> dsh;
            if (!mbar_wait(empty + s, (round & 1u) ^ 1u, limit)) { ok = false; return false; }
            uint32_t *slot = myring + (size_t)s * kSlotWords * 32;
            if (len < cnt) {
#pragma unroll
                for (int t = 0; t < 8; ++t) slot[32 * (kSlotP + t)] = pack_draw(r1[t], r3[t]);
            } else if (cnt == 8) {
                WinDec<MODE> d;
                decode_window<MODE, 8>(lat, cpb, L, WPR, row, q, half, r1, r3, nullptr, d);
                put_window<MODE, 8>(d, slot);
            } else {
                WinDec<MODE> d;
                decode_window<MODE, 4>(lat, cpb, L, WPR, row, q, half, r1, r3, nullptr, d);
                put_window<MODE, 4>(d, slot);
            }
            if (!silent) mbar_arrive(full + s);
            ++w;
            return true;
        });
    } else {
        const bool store = lane < cpb;
        ChainState st;
        st.E = cs.active ? a.edel[cs.chain] : (store ? 0 : 3);
        st.EJ = cs.active ? a.ej[cs.chain] : 0;
        st.M = (cs.active && MODE == kModeProduce) ? a.mag[cs.chain] : 0;
        const WT eps = (WT)a.log_eps;
        const bool checked = (unsigned long long)cpb * nup >= 0xFFFFFFFFull;
        for_each_window(L, WPR, a.therm, nup, [&](uint32_t row, uint32_t q, uint32_t half, uint32_t cnt,
                                                  uint32_t len, bool rec_phase) {
            const uint32_t s = w & (D - 1u), round = w >> dsh;
            if (!mbar_wait(full + s, round & 1u, limit)) { ok = false; return false; }
            const uint32_t *slot = myring + (size_t)s * kSlotWords * 32;
            const bool rec = rec_phase && cs.active;
            uint32_t *pc = lat + (size_t)(row * WPR + q) * cpb;
            if (len < cnt) {
                uint32_t p[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) p[t] = slot[32 * (kSlotP + t)];
                partial_core<MODE>(lat, cpb, L, WPR, row, q, half, len, rec, store, wP, histS, a.hist, st, p);
            } else if (cnt == 8) {
                WinDec<MODE> d;
                get_window<MODE, 8>(slot, pc, half, d);
                scan_window<MODE, 8, true>(d, rec, store, checked, wS, histS, a.hist, st, eps, wG, tol);
            } else {
                WinDec<MODE> d;
                get_window<MODE, 4>(slot, pc, half, d);
                scan_window<MODE, 4, true>(d, rec, store, checked, wS, histS, a.hist, st, eps, wG, tol);
            }
            mbar_arrive(empty + s);  // after the store: the producer may read the word
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
    uint32_t *lat = prologue<MODE, LAT_SMEM>(a, smem, lat_off, cpb, lane, blockIdx.x, wS, histS, gl);
    __syncthreads();
    ChainSetup<MODE, R> cs;
    cs.init(a, cpb, lane, blockIdx.x);
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

// The same against a table of logarithms (entry k for u = (2k+1) 2^-24).
__global__ void k_table_bracket(const float *tab, unsigned int *maxbits)
{
    unsigned int m = 0;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < (1u << 23); k += gridDim.x * blockDim.x) {
        const float u = u01f(k << 9);
        const float e = fabsf(__logf(u) - tab[k]);
        m = max(m, __float_as_uint(e));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxbits, m);
}

cudaError_t measure_table_bracket(const float *tab, float *max_abs_err, cudaStream_t s)
{
    unsigned int *d = nullptr, h = 0;
    cudaError_t e = cudaMalloc(&d, sizeof(unsigned int));
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(d, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) {
        k_table_bracket<<<152 * 8, 256, 0, s>>>(tab, d);
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

cudaError_t device_log_eps(int device, cudaStream_t s, double *eps)
{
    static std::mutex mu;
    static float maxerr[64];
    static bool have[64];
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!have[device]) {
        const cudaError_t e = measure_logf_bracket(&maxerr[device], s);
        if (e != cudaSuccess) return e;
        have[device] = true;
    }
    const float m = maxerr[device];
    *eps = (m >= 0.0f && m < 1e-2f) ? 2.0 * (double)m + 1e-30 : 1e30;
    return cudaSuccess;
}

// ---------------------------------------------------------------------------
SweepPlan plan_sweep(int mode, int rounds, uint32_t L, uint32_t nchains, size_t smem_optin, int sms, int kernel)
{
    SweepPlan p{};
    // every mode and placement defaults to the windowed kernel: with its
    // walk over whole row-halves it is also the faster one in production
    // with the lattice in global memory (146 against 136 attempts/ns for the
    // warp-specialised kernel at L=128, 142 against 138 at L=96, bit for bit
    // the same)
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
    // keep 512 B of the opt-in limit for the kernels' static shared memory
    const size_t optin = smem_optin > 512 ? smem_optin - 512 : 0;
    const size_t cap = optin > fixed ? (optin - fixed) / per_chain : 0;
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
    // a lattice in global memory: the windowed kernel keeps a four-row ring
    // per lane in shared memory when it fits
    p.row_ring = !p.lat_smem && p.kernel == kKernelWindowed && L % 4 == 0 && WPR <= 8 &&
                 base + ring_bytes(L, cpb) <= optin;
    p.smem = base + (p.kernel == kKernelSpecialized ? smem_ring_bytes(warps) : 0) +
             (p.lat_smem ? per_chain * cpb : 0) + (p.row_ring ? ring_bytes(L, cpb) : 0);
    return p;
}

template <int MODE, int R, bool LS>
static cudaError_t launch_one(const SweepPlan &p, const SweepArgs &a, cudaStream_t s)
{
    void (*kern)(const SweepArgs, uint32_t) =
        p.kernel == kKernelSpecialized ? k_sweep_spec<MODE, R, LS>
        : p.kernel == kKernelWindowed  ? (!LS && p.row_ring ? k_sweep_win<MODE, R, false, true> : k_sweep_win<MODE, R, LS>)
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
