// k_sweep_random.cu -- the random-site Metropolis sweep of the reference's
// CPU weight program (muca_mag.cpp:312-393, `mcs`) and of the GPU kernel
// mcs2 it was ported to (muca_delta_multigpu.cu:637-734), one chain per lane.
//
// Per chain (the reference's MPI rank WORKER, `seed` = jack index mm):
//   keys  k1 = {10 W + 1000 seed, 0xdecafbad}    (acceptance)
//         k2 = {100 W + 4000 seed, 0x20202041}   (site)
//         k3 = {1000 W + 10000 seed, 0x11cafead} (direction)
//   ctr   {c0, 0xbadbad11, 2 iter, 0xBADC0DED}, ++c0 before every 4th attempt,
//         continuing from the thermalisation into the production loop;
//   site  idx = (unsigned)(u01fixedpt<float>(r2) * N), truncated;
//   step  the same proposal and energy change as the sweep kernels, with
//         FP64 weights: diff = (double)(-2 dE) + w[E + dDel] - w[E];
//   test  diff >= 0 || log(u01fixedpt<float>(r1)) < diff, where log is the
//         host libm's logf (the CPU program) when a table of its values is
//         given, else CUDA's logf (mcs2).
// The lattice uses the packed layout of the other sweeps (2-bit codes, rows
// of 16-site words, [block][word][lane]); the FP32 difference table of the
// FP64 weights (stage_diff_table) and a u32 histogram are staged in shared
// memory, the lattice too when it fits.
//
// FP64 issues slowly on this GPU, and the exact log is a table lookup in
// global memory (host libm values) or a full logf: both used to sit on every
// attempt's dependency chain.  The test is decided in FP32 instead, as the
// production scan does it: log(u) < 0 for every u <= 1 - 2^-24, so the
// reference's test is  log(u) < diff;  with fast = -2 dE + T[E].(dDel)
// within tol of the FP64 diff and __logf(u) within `log_eps` of the exact
// log (measured over every u: against CUDA's logf, or against the host
// table), g = __logf(u) - fast has the sign of log(u) - diff whenever
// |g| > tol + log_eps.  Otherwise that lane forms the reference's FP64 diff
// from the global weights and the exact log, so every decision is the
// reference's.
#include "sweep_core.cuh"

#include <algorithm>

namespace muca {

// shared memory: the difference table (float2 per bin) | u32 histogram | lattice
__host__ __device__ inline size_t random_smem_base(uint32_t N)
{
    return align16((size_t)(N + 1) * 8) + align16((size_t)(N + 1) * 4);
}

template <int R, bool LAT_SMEM>
__global__ void __launch_bounds__(256) k_sweep_random(const RandomArgs a, uint32_t cpb)
{
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t iter = a.iter;
    unsigned long long nup = a.nup;
    if (a.dyn) {
        if (a.dyn[2]) return;
        iter = a.dyn[0];
        nup = a.dyn[1];
    }
    const uint32_t N = a.N, L = a.L, WPR = a.WPR, nt = blockDim.x, tid = threadIdx.x, lane = threadIdx.x;
    float2 *T = reinterpret_cast<float2 *>(smem);
    uint32_t *histS = reinterpret_cast<uint32_t *>(smem + align16((size_t)(N + 1) * 8));
    uint32_t *latS = reinterpret_cast<uint32_t *>(smem + random_smem_base(N));
    const double *__restrict__ w64 = a.w;
    const float band = stage_diff_table(w64, N, T) + (float)a.log_eps;
    for (uint32_t i = tid; i <= N; i += nt) histS[i] = 0u;
    const uint32_t words = L * WPR;
    const bool store = lane < cpb;
    const uint32_t l = store ? lane : 0u;
    uint32_t *gl = a.lat + (size_t)blockIdx.x * words * cpb + l;
    uint32_t *lat = gl;
    if (LAT_SMEM) {
        if (store)
            for (uint32_t w = 0; w < words; ++w) latS[(size_t)w * cpb + lane] = gl[(size_t)w * cpb];
        lat = latS + l;
    }
    __syncthreads();
    const uint32_t chain = blockIdx.x * cpb + lane;
    const bool active = store && chain < a.nchains;
    const uint32_t W = a.worker0 + chain;
    RoundKeys<R> k1, k2, k3;
    k1.init(10u * W + 1000u * a.seed, 0xdecafbadu);
    k2.init(100u * W + 4000u * a.seed, 0x20202041u);
    k3.init(1000u * W + 10000u * a.seed, 0x11cafeadu);
    // lanes of the last block past the chain count sweep their zero lattice
    // (E_Delta 0) and never record; padding lanes (>= cpb) read lane 0's
    // spins but never accept, so their E_Delta stays 1 and every weight
    // index E + dDel stays in [0, 2]
    int E = active ? a.edel[chain] : (store ? 0 : 1);
    int EJ = active ? a.ej[chain] : 0;
    const float fN = (float)N;
    uint32_t c0 = 0;
    uint4 r1 = make_uint4(0, 0, 0, 0), r2 = r1, r3 = r1;
    auto code_at = [&](uint32_t row, uint32_t col) -> uint32_t {
        return spin_code(lat[(size_t)(row * WPR + (col >> 4)) * cpb], col);
    };
    for (int phase = 0; phase < 2; ++phase) {
        const unsigned long long n = phase ? nup : a.therm;
        for (unsigned long long i = 0; i < n; ++i) {
            const int sub = (int)(i & 3ull);
            if (sub == 0) {
                ++c0;
                r1 = philox<R>(c0, 0xbadbad11u, 2u * iter, kCtrTag, k1);
                r2 = philox<R>(c0, 0xbadbad11u, 2u * iter, kCtrTag, k2);
                r3 = philox<R>(c0, 0xbadbad11u, 2u * iter, kCtrTag, k3);
            }
            const uint32_t idx = __float2uint_rz(__fmul_rn(u01f(pick(r2, sub)), fN));
            // idx / L as a high product with ceil(2^32 / L): exact for idx < 2^16
            // and L <= 128 (the rounding error idx / 2^32 < 1/L)
            const uint32_t row = __umulhi(idx, a.inv_L), col = idx - row * L;
            uint32_t *pw = lat + (size_t)(row * WPR + (col >> 4)) * cpb;
            const int os = (int)spin_code(*pw, col) - 1;
            int ns = os + ((pick(r3, sub) >> 31) ? -1 : 1);  // u01fixedpt<float>(r3) < 0.5 <=> top bit clear
            ns = ns - 3 * (ns == 2) + 3 * (ns == -2);
            const uint32_t cl = col ? col - 1 : L - 1, cr = (col + 1 == L) ? 0u : col + 1;
            const uint32_t ru = (row + 1 == L) ? 0u : row + 1, rd = row ? row - 1 : L - 1;
            const int nb = (int)(code_at(row, cl) + code_at(row, cr) + code_at(ru, col) + code_at(rd, col)) - 4;
            const int tmp = ns * (os == 0) + os;  // the trial value the reference stores before forming dE
            const int dE = ((os == 0) + os * (ns - os)) * (-tmp) * nb;
            const int dDel = ns * ns - os * os;
            const uint32_t r = pick(r1, sub);
            const float2 tE = T[E];
            const float dl = dDel == 0 ? 0.0f : (dDel < 0 ? tE.x : tE.y);
            const float g = __fsub_rn(__logf(u01f(r)), __fadd_rn(small_int_to_float(-2 * dE), dl));
            bool acc = g < 0.0f;
            if (fabsf(g) <= band) {
                // in doubt: the reference's FP64 difference and exact log
                const double diff = __dsub_rn(__dadd_rn((double)(-dE * 2), w64[E + dDel]), w64[E]);
                acc = diff >= 0.0;
                if (!acc) {
                    const float lg = a.logf_tab ? __ldg(a.logf_tab + (r >> 9)) : logf(u01f(r));
                    acc = (double)lg < diff;
                }
            }
            if (acc && store) {
                const uint32_t sh = 2u * (col & 15u);
                *pw = (*pw & ~(3u << sh)) | ((uint32_t)(ns + 1) << sh);
                EJ += dE;
                E += dDel;
            }
            if (phase == 1 && active) {
                // a u32 shared bin is drained into the u64 device bin at 2^31
                const uint32_t old = atomicAdd(&histS[E], 1u);
                if (old >= 0x80000000u) atomicAdd(&a.hist[E], (unsigned long long)atomicExch(&histS[E], 0u));
            }
        }
    }
    if (LAT_SMEM && store) {
        for (uint32_t w = 0; w < words; ++w) gl[(size_t)w * cpb] = lat[(size_t)w * cpb];
    }
    if (active) {
        a.edel[chain] = E;
        a.ej[chain] = EJ;
    }
    __syncthreads();
    for (uint32_t b = tid; b <= N; b += nt) {
        const uint32_t v = histS[b];
        if (v) atomicAdd(&a.hist[b], (unsigned long long)v);
    }
}

template <int R, bool LS>
static cudaError_t launch_random_one(const RandomArgs &a, uint32_t cpb, uint32_t blocks, size_t smem, cudaStream_t s)
{
    const cudaError_t e = cudaFuncSetAttribute(k_sweep_random<R, LS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem);
    if (e != cudaSuccess) return e;
    k_sweep_random<R, LS><<<blocks, (cpb + 31u) / 32u * 32u, smem, s>>>(a, cpb);
    return cudaGetLastError();
}

// Block shape of the random-site sweep: one wave of blocks over the SMs with
// the chains spread evenly (ceil(nchains / SMs) per block), each block's
// lattice in shared memory when that many chains' lattices fit beside the
// difference table and the histogram.  The random site makes the lattice
// loads of one attempt depend on the previous attempt's store, so their
// latency is on every attempt's chain: shared memory, not L1/L2.  When the
// lattices do not fit, blocks of up to 128 chains read them from global
// memory.
SweepPlan plan_random(uint32_t L, uint32_t nchains, size_t smem_optin, int sms)
{
    SweepPlan p{};
    p.mode = kModeWeight;
    p.kernel = kKernelGeneric;
    const uint32_t N = L * L, WPR = (L + 15) / 16;
    const size_t per_chain = (size_t)L * WPR * 4, base = random_smem_base(N);
    const size_t optin = smem_optin > 512 ? smem_optin - 512 : 0;
    const size_t cap = optin > base ? (optin - base) / per_chain : 0;
    const uint32_t want = (nchains + (uint32_t)sms - 1) / (uint32_t)sms;
    p.lat_smem = cap >= 1 && want <= cap && want <= 256;
    p.cpb = p.lat_smem ? want : std::min<uint32_t>(128u, want);
    p.blocks = (nchains + p.cpb - 1) / p.cpb;
    p.threads = (p.cpb + 31u) / 32u * 32u;
    p.smem = random_sweep_smem(L, p.cpb, p.lat_smem);
    return p;
}

size_t random_sweep_smem(uint32_t L, uint32_t cpb, bool lat_smem)
{
    const uint32_t WPR = (L + 15) / 16;
    return random_smem_base(L * L) + (lat_smem ? (size_t)L * WPR * 4 * cpb : 0);
}

cudaError_t launch_sweep_random(const RandomArgs &a, uint32_t cpb, uint32_t blocks, int rounds, size_t smem_optin,
                                cudaStream_t s)
{
    if (cpb == 0 || cpb > 256 || a.L < 3) return cudaErrorInvalidValue;
    // (512 B of the opt-in limit stay free for the kernel's static shared memory)
    const bool ls = random_sweep_smem(a.L, cpb, true) + 512 <= smem_optin;
    const size_t smem = random_sweep_smem(a.L, cpb, ls);
    if (smem > smem_optin) return cudaErrorInvalidValue;
    if (rounds == 10)
        return ls ? launch_random_one<10, true>(a, cpb, blocks, smem, s) : launch_random_one<10, false>(a, cpb, blocks, smem, s);
    return ls ? launch_random_one<7, true>(a, cpb, blocks, smem, s) : launch_random_one<7, false>(a, cpb, blocks, smem, s);
}

}  // namespace muca
