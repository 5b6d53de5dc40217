// k_lattice.cu -- chain initialisation and lattice (un)packing on the device.
//
// The reference initialises every chain's lattice on the host, one Philox
// block per 4 sites, then copies it to the device and runs computeEnergies /
// computeDeltaE (/computeM) (muca_delta_multigpu.cu:340-359,
// produce2_multigpu.cu:126-140,272-274).  Here one thread builds one packed
// 16-site word of one chain directly in device memory (the Philox stream of
// a site is a pure function of (chain, site), so words are independent), and
// a second kernel forms E_J, E_Delta and M per chain.
#include "muca_device.cuh"
#include "muca_internal.h"

namespace muca {

template <int R>
__device__ __forceinline__ uint4 init_block(const InitArgs &ia, uint32_t W, uint32_t dev, uint32_t chain,
                                            uint32_t jack, uint32_t g)
{
    RoundKeys<R> k;
    uint32_t c[4];
    k.init(ia.key0_mul * W + ia.key0_jack_mul * jack + ia.key0_add, ia.key1 + ia.key1_jack_mul * jack);
    if (ia.chain_in_ctr) {
        c[0] = ia.chain_offset + chain; c[1] = g; c[2] = 0; c[3] = 0;
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) c[j] = ia.ctr0[j] + ia.ctr0_dev_mul[j] * dev;
        c[ia.ctr_word] += g + 1u;  // ++c[word] before every 4th site
    }
    return philox<R>(c[0], c[1], c[2], c[3], k);
}

template <int R>
__global__ void k_init(uint32_t *lat, uint32_t L, uint32_t WPR, uint32_t cpb, uint32_t nchains,
                       uint32_t chains_per_dev, uint32_t jack, InitArgs ia)
{
    const uint32_t words = L * WPR;
    const size_t total = (size_t)((nchains + cpb - 1) / cpb) * cpb * words;
    const bool narrow = total <= 0xFFFFFFFFull;  // 32-bit index arithmetic (uniform)
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        // t enumerates [block][word][lane] exactly like the packed layout
        uint32_t lane, w, blk;
        if (narrow) {
            const uint32_t t32 = (uint32_t)t, bw = t32 / cpb;
            lane = t32 - bw * cpb;
            blk = bw / words;
            w = bw - blk * words;
        } else {
            const size_t bw = t / cpb;
            lane = (uint32_t)(t - bw * cpb);
            blk = (uint32_t)(bw / words);
            w = (uint32_t)(bw - (size_t)blk * words);
        }
        const uint32_t chain = blk * cpb + lane;
        uint32_t word = kZeroWord;
        if (chain < nchains) {
            const uint32_t dev = chain / chains_per_dev, W = chain - dev * chains_per_dev;
            const uint32_t row = w / WPR, q = w - row * WPR;
            const uint32_t c_lo = 16u * q, c_hi = min(16u * q + 16u, L);
            word = 0;
            uint32_t g_cur = 0xFFFFFFFFu;
            uint4 r = make_uint4(0, 0, 0, 0);
            for (uint32_t col = c_lo; col < c_hi; ++col) {
                int s;
                if (ia.ordered) {
                    s = 1;
                } else {
                    const uint32_t site = row * L + col, g = site >> 2;
                    if (g != g_cur) {
                        r = init_block<R>(ia, W, dev, chain, jack, g);
                        g_cur = g;
                    }
                    const uint32_t rw = pick(r, (int)(site & 3u));
                    s = ia.graded ? graded_spin(rw, W, chains_per_dev) : init_spin(rw);
                }
                word |= (uint32_t)(s + 1) << (2u * (col - c_lo));
            }
        }
        lat[t] = word;
    }
}

__global__ void k_pack(uint32_t *lat, const int8_t *src, uint32_t L, uint32_t WPR, uint32_t cpb, uint32_t nchains)
{
    const uint32_t words = L * WPR;
    const size_t total = (size_t)((nchains + cpb - 1) / cpb) * cpb * words;
    const size_t N = (size_t)L * L;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const uint32_t lane = (uint32_t)(t % cpb);
        const size_t bw = t / cpb;
        const uint32_t w = (uint32_t)(bw % words);
        const uint32_t chain = (uint32_t)(bw / words) * cpb + lane;
        uint32_t word = kZeroWord;
        if (chain < nchains) {
            const uint32_t row = w / WPR, q = w - row * WPR;
            const uint32_t c_lo = 16u * q, c_hi = min(16u * q + 16u, L);
            const int8_t *p = src + chain * N + (size_t)row * L;
            word = 0;
            for (uint32_t col = c_lo; col < c_hi; ++col) word |= (uint32_t)(p[col] + 1) << (2u * (col - c_lo));
        }
        lat[t] = word;
    }
}

__global__ void k_unpack(const uint32_t *lat, int8_t *dst, uint32_t L, uint32_t WPR, uint32_t cpb, uint32_t nchains)
{
    const uint32_t words = L * WPR;
    const size_t total = (size_t)((nchains + cpb - 1) / cpb) * cpb * words;
    const size_t N = (size_t)L * L;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const uint32_t lane = (uint32_t)(t % cpb);
        const size_t bw = t / cpb;
        const uint32_t w = (uint32_t)(bw % words);
        const uint32_t chain = (uint32_t)(bw / words) * cpb + lane;
        if (chain >= nchains) continue;
        const uint32_t row = w / WPR, q = w - row * WPR;
        const uint32_t c_lo = 16u * q, c_hi = min(16u * q + 16u, L);
        const uint32_t word = lat[t];
        int8_t *p = dst + chain * N + (size_t)row * L;
        for (uint32_t col = c_lo; col < c_hi; ++col) p[col] = (int8_t)((int)spin_code(word, col) - 1);
    }
}

// E_J = -sum over bonds (right and up neighbour of every site), which equals
// total_energy of muca_delta_multigpu.cu:563-571 (the sum over all four
// neighbours, halved), E_Delta = sum s^2, M = sum s.
__global__ void k_energies(const uint32_t *lat, int32_t *ej, int32_t *edel, int32_t *mag, uint32_t L, uint32_t WPR,
                           uint32_t cpb, uint32_t nchains)
{
    const uint32_t chain = blockIdx.x * blockDim.x + threadIdx.x;
    if (chain >= nchains) return;
    const uint32_t words = L * WPR;
    const uint32_t *base = lat + (size_t)(chain / cpb) * words * cpb + (chain % cpb);
    auto get = [&](uint32_t r, uint32_t c) -> int {
        return (int)spin_code(base[(size_t)(r * WPR + (c >> 4)) * cpb], c) - 1;
    };
    int bonds = 0, d = 0, m = 0;
    for (uint32_t r = 0; r < L; ++r) {
        const uint32_t ru = (r + 1 == L) ? 0 : r + 1;
        for (uint32_t c = 0; c < L; ++c) {
            const int s = get(r, c);
            const uint32_t cr = (c + 1 == L) ? 0 : c + 1;
            bonds += s * (get(r, cr) + get(ru, c));
            d += s * s;
            m += s;
        }
    }
    ej[chain] = -bonds;
    edel[chain] = d;
    if (mag) mag[chain] = m;
}

__global__ void k_validate(const int8_t *src, size_t n, unsigned long long *bad)
{
    unsigned long long cnt = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int v = src[i];
        cnt += (v < -1 || v > 1);
    }
    if (cnt) atomicAdd(bad, cnt);
}

static unsigned grid_for(size_t total)
{
    size_t g = (total + 255) / 256;
    return (unsigned)(g > 65535 * 8 ? 65535 * 8 : (g ? g : 1));
}

cudaError_t launch_init(uint32_t *lat, uint32_t L, uint32_t WPR, uint32_t cpb, uint32_t nchains,
                        uint32_t chains_per_dev, uint32_t jack, const InitArgs &ia, cudaStream_t s)
{
    const size_t total = (size_t)((nchains + cpb - 1) / cpb) * cpb * L * WPR;
    if (ia.rounds == 10)
        k_init<10><<<grid_for(total), 256, 0, s>>>(lat, L, WPR, cpb, nchains, chains_per_dev, jack, ia);
    else
        k_init<7><<<grid_for(total), 256, 0, s>>>(lat, L, WPR, cpb, nchains, chains_per_dev, jack, ia);
    return cudaGetLastError();
}

cudaError_t launch_pack(uint32_t *lat, const int8_t *src, uint32_t L, uint32_t WPR, uint32_t cpb, uint32_t nchains,
                        cudaStream_t s)
{
    const size_t total = (size_t)((nchains + cpb - 1) / cpb) * cpb * L * WPR;
    k_pack<<<grid_for(total), 256, 0, s>>>(lat, src, L, WPR, cpb, nchains);
    return cudaGetLastError();
}

cudaError_t launch_unpack(const uint32_t *lat, int8_t *dst, uint32_t L, uint32_t WPR, uint32_t cpb,
                          uint32_t nchains, cudaStream_t s)
{
    const size_t total = (size_t)((nchains + cpb - 1) / cpb) * cpb * L * WPR;
    k_unpack<<<grid_for(total), 256, 0, s>>>(lat, dst, L, WPR, cpb, nchains);
    return cudaGetLastError();
}

cudaError_t launch_energies(const uint32_t *lat, int32_t *ej, int32_t *edel, int32_t *mag, uint32_t L, uint32_t WPR,
                            uint32_t cpb, uint32_t nchains, cudaStream_t s)
{
    k_energies<<<(nchains + 127) / 128, 128, 0, s>>>(lat, ej, edel, mag, L, WPR, cpb, nchains);
    return cudaGetLastError();
}

cudaError_t launch_validate(const int8_t *src, size_t n, unsigned long long *bad, cudaStream_t s)
{
    k_validate<<<grid_for(n), 256, 0, s>>>(src, n, bad);
    return cudaGetLastError();
}

}  // namespace muca
