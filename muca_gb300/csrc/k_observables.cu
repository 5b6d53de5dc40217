// k_observables.cu -- production reweighting on the device, FP64.
//
// Replaces the host code of the reference production program that runs per
// Delta point: weight_shift (produce2_multigpu.cu:391-400), the Boltzmann
// factors boltz_j = exp(-beta*delta*j - lnW_j) (:297), the reweighting sums
// over the triangular (E_Delta, M) histogram (observables, :498-518; the
// reference sums in x87 long double on the host) and the jackknife
// (:520-535).  The triangle's row i (E_Delta = i) holds the i+1 bins
// m = -i, -i+2, ..., i at (i^2 + 2i + m)/2 = i(i+1)/2 + (m+i)/2.
//
// The sums stream the u64 histogram once (HBM bound at 8 B per bin), one
// warp per row, with exact integer moments per row (see k_observables);
// the per-row FP64 terms are combined per warp, per block and then in a
// fixed-order second pass, so the result is deterministic and agrees with
// the long-double host sum to ~1e-15.
#include "muca_device.cuh"
#include "muca_internal.h"

#include <mutex>

namespace muca {

constexpr int kObsThreads = 256;
// 2 blocks per SM are resident (96 registers per thread), so the grid is one
// wave of them over the 152 SMs of GB300 (measured: 12 % faster at L=96 than
// two waves of 608 blocks)
constexpr int kObsBlocks = 152 * 2;

__global__ void k_weight_shift(double *lnw, uint32_t N, double beta, double delta)
{
    __shared__ double sh[32];
    const double bd = __dmul_rn(beta, delta);
    double mx = -1.0 / 0.0;
    for (uint32_t i = threadIdx.x; i <= N; i += blockDim.x) {
        const double v = __dsub_rn(-lnw[i], __dmul_rn(bd, (double)i));
        mx = v > mx ? v : mx;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { const double t = __shfl_xor_sync(0xffffffffu, mx, o); mx = t > mx ? t : mx; }
    if (lane == 0) sh[wid] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = sh[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = sh[w] > m ? sh[w] : m;
        sh[0] = m;
    }
    __syncthreads();
    const double m = sh[0];
    for (uint32_t i = threadIdx.x; i <= N; i += blockDim.x) lnw[i] = __dadd_rn(lnw[i], m);
}

// One warp per row of the triangle at a time (row i = E_Delta holds the i+1
// bins m = -i, -i+2, ..., i from b = i(i+1)/2): the lanes stream the row's
// u64 counts with coalesced loads, 2 kObsUnroll independent loads per lane
// in flight (double-buffered).  Within a row boltz_i is a common factor, so the lanes sum
// H, |m| H, m^2 H and m^4 H exactly in 128-bit integers (integer pipes; FP64
// issues slowly on this GPU), the warp reduces them, and lane 0 adds
// sum_k(i) * boltz_i to its FP64 accumulators: one FP64 product per row and
// moment instead of one per bin.  Warp w takes rows w, w + W, w + 2W, ...
// (W warps in the grid), which spreads the long rows evenly.
constexpr int kObsUnroll = 8;

typedef unsigned __int128 u128;

__device__ __forceinline__ u128 shfl_xor_u128(u128 v, int o)
{
    const unsigned long long lo = __shfl_xor_sync(0xffffffffu, (unsigned long long)v, o);
    const unsigned long long hi = __shfl_xor_sync(0xffffffffu, (unsigned long long)(v >> 64), o);
    return ((u128)hi << 64) | lo;
}

__device__ __forceinline__ double u128_to_double(u128 v)
{
    return __dadd_rn(__dmul_rn((double)(unsigned long long)(v >> 64), 18446744073709551616.0),
                     (double)(unsigned long long)v);
}

__global__ void __launch_bounds__(kObsThreads) k_observables(const unsigned long long *__restrict__ hist,
                                                             const double *__restrict__ lnw, uint32_t N,
                                                             double beta, double delta,
                                                             double *__restrict__ partials)
{
    const double nbd = __dmul_rn(-beta, delta);
    double s0 = 0, s1 = 0, s2 = 0, s4 = 0;
    const uint32_t ln = threadIdx.x & 31u;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i <= N; i += nwarps) {
        const unsigned long long *row = hist + (unsigned long long)i * (i + 1) / 2;
        u128 a0 = 0, a1 = 0, a2 = 0, a4 = 0;
        // double-buffered: the next chunk's loads are in flight while this one is summed
        unsigned long long h[kObsUnroll], hn[kObsUnroll];
#pragma unroll
        for (int k = 0; k < kObsUnroll; ++k) {
            const uint32_t j = ln + 32u * k;
            h[k] = j <= i ? __ldcs(row + j) : 0ull;
        }
        for (uint32_t j0 = 0; j0 <= i; j0 += 32u * kObsUnroll) {
#pragma unroll
            for (int k = 0; k < kObsUnroll; ++k) {
                const uint32_t j = j0 + 32u * kObsUnroll + ln + 32u * k;
                hn[k] = j <= i ? __ldcs(row + j) : 0ull;
            }
#pragma unroll
            for (int k = 0; k < kObsUnroll; ++k) {
                const unsigned long long H = h[k];
                const int m = 2 * (int)(j0 + ln + 32u * k) - (int)i;
                const uint32_t am = (uint32_t)(m < 0 ? -m : m);  // <= N <= 16384
                const uint32_t am2 = am * am;                    // < 2^29
                // 64 x 32-bit products; H m^4 = (H m^2) m^2 with H m^2 < 2^93
                const u128 t = (u128)H * am2;
                const unsigned long long tl = (unsigned long long)t, th = (unsigned long long)(t >> 64);
                a0 += H;
                a1 += (u128)H * am;
                a2 += t;
                a4 += (u128)tl * am2 + ((u128)(th * am2) << 64);
            }
#pragma unroll
            for (int k = 0; k < kObsUnroll; ++k) h[k] = hn[k];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a0 += shfl_xor_u128(a0, o);
            a1 += shfl_xor_u128(a1, o);
            a2 += shfl_xor_u128(a2, o);
            a4 += shfl_xor_u128(a4, o);
        }
        if (ln == 0 && a0 != 0) {
            const double bz = exp(__dsub_rn(__dmul_rn(nbd, (double)i), lnw[i]));
            s0 = __dadd_rn(s0, __dmul_rn(u128_to_double(a0), bz));
            s1 = __dadd_rn(s1, __dmul_rn(u128_to_double(a1), bz));
            s2 = __dadd_rn(s2, __dmul_rn(u128_to_double(a2), bz));
            s4 = __dadd_rn(s4, __dmul_rn(u128_to_double(a4), bz));
        }
    }
    __shared__ double sh[4][kObsThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        s4 += __shfl_xor_sync(0xffffffffu, s4, o);
    }
    if (lane == 0) { sh[0][wid] = s0; sh[1][wid] = s1; sh[2][wid] = s2; sh[3][wid] = s4; }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0;
        for (int w = 0; w < kObsThreads / 32; ++w) t += sh[threadIdx.x][w];
        partials[(size_t)blockIdx.x * 4 + threadIdx.x] = t;
    }
}

__global__ void k_observables_final(const double *partials, int nblocks, double *out)
{
    if (threadIdx.x < 4) {
        double t = 0;
        for (int b = 0; b < nblocks; ++b) t += partials[(size_t)b * 4 + threadIdx.x];
        out[threadIdx.x] = t;
    }
}

// jakknife (muca_delta_multigpu.cu:620-635), one thread, same order.
__global__ void k_jackknife(const double *x, uint32_t J, double *out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double avg = 0;
    for (uint32_t i = 0; i < J; i++) avg += x[i];
    const double total = avg;
    avg = avg / (double)J;
    double dev = 0;
    for (uint32_t i = 0; i < J; i++) {
        const double mi = (total - x[i]) / (double)(J - 1);
        dev += (avg - mi) * (avg - mi);
    }
    dev = (double)(J - 1) * dev / (double)J;
    out[0] = avg;
    out[1] = sqrt(dev);
}

cudaError_t launch_weight_shift(double *lnw, uint32_t N, double beta, double delta, cudaStream_t s)
{
    k_weight_shift<<<1, 1024, 0, s>>>(lnw, N, beta, delta);
    return cudaGetLastError();
}

size_t observables_partials(uint32_t) { return (size_t)kObsBlocks * 4; }

cudaError_t launch_observables(const unsigned long long *hist2d, const double *lnw, uint32_t N, double beta,
                               double delta, double *partials, double *out, cudaStream_t s)
{
    k_observables<<<kObsBlocks, kObsThreads, 0, s>>>(hist2d, lnw, N, beta, delta, partials);
    k_observables_final<<<1, 32, 0, s>>>(partials, kObsBlocks, out);
    return cudaGetLastError();
}

cudaError_t launch_jackknife(const double *x, uint32_t n, double *out2, cudaStream_t s)
{
    k_jackknife<<<1, 32, 0, s>>>(x, n, out2);
    return cudaGetLastError();
}

// ---- the reweighting sums without any allocation ------------------------
//
// Some callers cannot let this library allocate device memory.  Example: a
// scheduler that packs many production instances into a fixed HBM budget
// through its own pool, where a hidden cudaMalloc would break the budget and
// also synchronise the device under the scheduler's other streams.  Another:
// a process that only reweights histograms it already holds on the device.
// It has no lattice and so no engine context, whose creation allocates.  For
// them, the two kernels above run with their block partials in the
// file-scope array below instead of context memory.
//
// The array holds the partials of the fixed kObsBlocks-block grid,
// kObsBlocks x 4 doubles (9,728 bytes), whatever L is.  Each block
// overwrites its own four entries before the final pass reads them, so
// nothing in it has to start at zero, and no state carries from one call to
// the next.  There is one array per device, shared by every caller in the
// process: two calls in flight at once on the same device (two streams, or
// two host threads) write the same entries and race.
constexpr size_t kStaticPartials = (size_t)kObsBlocks * 4;
static __device__ __align__(256) double g_obs_partials[kStaticPartials];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_partials_mu;
double *g_partials_addr[kMaxDevices] = {};
}  // namespace

size_t observables_static_partials() { return kStaticPartials; }

cudaError_t launch_observables_static(int device, const unsigned long long *hist2d, const double *lnw, uint32_t N,
                                      double beta, double delta, double *out, cudaStream_t s)
{
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    if (observables_partials(N) > kStaticPartials) return cudaErrorInvalidValue;
    double *partials = nullptr;
    {
        // The address is resolved once per device, with that device current
        // (the caller has made it current).  The first resolution may load
        // this module onto the device.
        std::lock_guard<std::mutex> lock(g_partials_mu);
        if (!g_partials_addr[device]) {
            void *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_obs_partials);
            if (e != cudaSuccess) return e;
            g_partials_addr[device] = static_cast<double *>(p);
        }
        partials = g_partials_addr[device];
    }
    return launch_observables(hist2d, lnw, N, beta, delta, partials, out, s);
}

}  // namespace muca
