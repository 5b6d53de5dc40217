// k_bench.cu -- measurement kernels for the rooflines of the sweep.
//
// The sweep kernels spend most of their issue slots on Philox4x32 blocks
// (two per four Metropolis attempts).  k_philox_peak generates Philox blocks
// in exactly the form the sweeps use them (per-thread key, counter words 1..3
// fixed, word 0 counting) at full occupancy with nothing else to do, so its
// rate is the ceiling of "Philox blocks per second" on this GPU.
//
// k_sweep_floor takes the weight-mode windowed sweep apart and times each
// part per warp in SM cycles (clock64), in the sweep's own geometry at
// 16384 chains: one block of four warps of 32 chains on one SM, one warp per
// SM sub-partition, the L = 72 lattice, the FP32 weights and the u32
// histogram in shared memory (225,824 B).  Each lane runs `windows` full
// 8-site windows:
//   part 0  the sweep's window body: the next window's draws, decode, scan,
//           lattice store and histogram entries (the sweep without its
//           4-site and partial windows and its loop bookkeeping);
//   part 1  the draws and the decode alone, the work off the chain of
//           decisions (its fields folded into one word so none is dead);
//   part 2  the scan, store and histogram entries alone, on two decoded
//           windows held in registers;
//   part 3  the bare chain of decisions of the scan: per attempt a select of
//           the prefetched weight, two adds, one compare, the E_Delta update
//           and the two weight loads one attempt ahead, with the scan's
//           loads at each window start;
//   part 4  the draws alone (four Philox4x32-7 blocks per window);
//   part 5  one dependent FP32 add per "attempt" (its latency);
//   part 6  one dependent shared-memory load per "attempt" (its latency).
// Parts 2 and 3 replay fixed windows, so E_Delta is kept inside the weight
// array by walls: the weights at E_Delta = 0..2 and N-2..N are -1e30, every
// move onto them is rejected, and the loads reach at most three bins beyond
// the current E_Delta.
#include "sweep_core.cuh"

namespace muca {

template <int R>
__global__ void __launch_bounds__(256) k_philox_peak(uint32_t blocks_per_thread, uint32_t seed, uint32_t *out)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    RoundKeys<R> k;
    k.init(2u * t, 0xdecafbadu);
    uint32_t acc = 0;
#pragma unroll 4
    for (uint32_t i = 0; i < blocks_per_thread; ++i) {
        const uint4 r = philox<R>(i + 1u, seed, t, kCtrTag, k);
        acc ^= r.x ^ r.y ^ r.z ^ r.w;
    }
    out[t] = acc;
}

cudaError_t launch_philox_peak(int rounds, uint32_t grid, uint32_t blocks_per_thread, uint32_t *out, cudaStream_t s)
{
    if (rounds == 10)
        k_philox_peak<10><<<grid, 256, 0, s>>>(blocks_per_thread, 100u, out);
    else
        k_philox_peak<7><<<grid, 256, 0, s>>>(blocks_per_thread, 100u, out);
    return cudaGetLastError();
}

constexpr uint32_t kFloorL = 72, kFloorWPR = 5, kFloorCpb = 128, kFloorN = kFloorL * kFloorL;
constexpr float kFloorEps = 3.5e-6f;  // twice max |__logf(u) - logf(u)| measured on GB300

__device__ __forceinline__ uint32_t floor_hash(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

template <int PART>
__global__ void __launch_bounds__(kFloorCpb, 1) k_sweep_floor(uint32_t windows, unsigned long long *cycles,
                                                               uint32_t *sink, unsigned long long *hist_dummy)
{
    extern __shared__ __align__(16) unsigned char smem[];
    float *wS = reinterpret_cast<float *>(smem);
    uint32_t *histS = reinterpret_cast<uint32_t *>(smem + smem_weights_bytes(kModeWeight, kFloorN));
    const uint32_t lane = threadIdx.x;
    uint32_t *lat = reinterpret_cast<uint32_t *>(smem + smem_weights_bytes(kModeWeight, kFloorN) +
                                                 smem_hist_bytes(kModeWeight, kFloorN)) + lane;
    const bool walls = PART >= 2;
    for (uint32_t b = lane; b <= kFloorN; b += blockDim.x) {
        wS[b] = (walls && (b < 3 || b + 3 > kFloorN)) ? -1e30f : 0.0f;
        histS[b] = 0;
    }
    // random spin codes 0..2 in the L sites of each row, code 1 (spin 0) in the padding
    int E = 0;
    for (uint32_t w = 0; w < kFloorL * kFloorWPR; ++w) {
        const uint32_t q = w % kFloorWPR;
        uint32_t word = 0;
        for (uint32_t c = 0; c < 16; ++c) {
            const uint32_t code = (16 * q + c < kFloorL) ? floor_hash(w * 16 + c + 7919u * lane) % 3u : 1u;
            word |= code << (2 * c);
            E += code != 1u;
        }
        lat[(size_t)w * kFloorCpb] = word;
    }
    __syncthreads();
    ChainState st;
    st.E = walls ? (int)(kFloorN / 2) : E;
    st.EJ = 0;
    st.M = 0;
    RoundKeys<7> k1, k3;
    k1.init(2u * lane + 1u, 0xdecafbadu);
    k3.init(2u * lane + 3u, 0xdecafbadu);
    uint32_t n1[8], n3[8];
    draw_pair<7>(1u, 100u, 0u, k1, k3, n1, n3);
    draw_pair<7>(2u, 100u, 0u, k1, k3, n1 + 4, n3 + 4);
    uint32_t cc = 2, fold = 0;
    WinDec<kModeWeight> d0, d1;
    if (PART >= 2) {
        decode_window<kModeWeight, 8>(lat, kFloorCpb, kFloorL, kFloorWPR, 3, 1, 0, n1, n3, nullptr, d0);
        draw_pair<7>(3u, 100u, 0u, k1, k3, n1, n3);
        draw_pair<7>(4u, 100u, 0u, k1, k3, n1 + 4, n3 + 4);
        decode_window<kModeWeight, 8>(lat, kFloorCpb, kFloorL, kFloorWPR, 5, 2, 1, n1, n3, nullptr, d1);
    }
    // part 6: a permutation of the bins to chase through shared memory
    if (PART == 6)
        for (uint32_t b = lane; b <= kFloorN; b += blockDim.x) histS[b] = (b * 7u + 3u) % (kFloorN + 1u);
    __syncthreads();
    float fx = 1.0f + u01f(n1[0]), fy = u01f(n1[1]);
    int ix = (int)(n1[2] % (kFloorN + 1u));
    const unsigned long long t0 = clock64();
    if (PART == 4) {
#pragma unroll 1
        for (uint32_t k = 0; k < windows; ++k) {
            draw_pair<7>(cc + 1, 100u, 0u, k1, k3, n1, n3);
            draw_pair<7>(cc + 2, 100u, 0u, k1, k3, n1 + 4, n3 + 4);
            cc += 2;
#pragma unroll
            for (int t = 0; t < 8; ++t) fold ^= n1[t] + n3[t];
        }
    } else if (PART == 5) {
#pragma unroll 1
        for (uint32_t k = 0; k < windows; ++k) {
#pragma unroll
            for (int t = 0; t < 8; ++t) fx = __fadd_rn(fx, fy);
        }
        fold = __float_as_uint(fx);
    } else if (PART == 6) {
#pragma unroll 1
        for (uint32_t k = 0; k < windows; ++k) {
#pragma unroll
            for (int t = 0; t < 8; ++t) ix = (int)histS[ix];
        }
        fold = (uint32_t)ix;
    } else if (PART <= 1) {
        uint32_t row = 0, q = 0, half = 0;
#pragma unroll 1
        for (uint32_t k = 0; k < windows; ++k) {
            uint32_t r1[8], r3[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                r1[t] = n1[t];
                r3[t] = n3[t];
            }
            draw_pair<7>(cc + 1, 100u, 0u, k1, k3, n1, n3);
            draw_pair<7>(cc + 2, 100u, 0u, k1, k3, n1 + 4, n3 + 4);
            cc += 2;
            if (PART == 0) {
                window_core<kModeWeight, 8, -1>(lat, kFloorCpb, kFloorL, kFloorWPR, row, q, true, true, false, wS,
                                                histS, hist_dummy, st, r1, r3, kFloorEps, nullptr, half);
            } else {
                WinDec<kModeWeight> d;
                decode_window<kModeWeight, 8>(lat, kFloorCpb, kFloorL, kFloorWPR, row, q, half, r1, r3, nullptr, d);
                uint32_t f = d.C ^ d.vnib ^ (uint32_t)(size_t)d.pc;
#pragma unroll
                for (int t = 0; t < 8; ++t)
                    f ^= ((uint32_t)d.dE[t] + ((uint32_t)d.dDel[t] << 8)) ^ __float_as_uint(d.f2[t]) ^
                         __float_as_uint(d.lf[t]) ^ d.p[t];
                fold += f;
            }
            // the full windows of the L = 72 rows: words 0..3 of each row
            if (++q == 4) {
                q = 0;
                if (++row == kFloorL) { row = 0; half ^= 1u; }
            }
        }
    } else if (PART == 2) {
#pragma unroll 1
        for (uint32_t k = 0; k < windows; k += 2) {
            scan_window<kModeWeight, 8>(d0, true, true, false, wS, histS, hist_dummy, st, kFloorEps);
            scan_window<kModeWeight, 8>(d1, true, true, false, wS, histS, hist_dummy, st, kFloorEps);
        }
    } else if (PART == 3) {
        auto chain = [&](const WinDec<kModeWeight> &d) {
            float wE = wS[st.E];
            float A = wS[st.E + d.dDel[0]];
            float c0 = wS[st.E + d.dDel[1]], c1 = wS[st.E + d.dDel[0] + d.dDel[1]];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const float diff = __fsub_rn(__fadd_rn(d.f2[t], A), wE);
                const bool acc = d.lf[t] < diff;
                if (acc) {
                    st.E += d.dDel[t];
                    wE = A;
                }
                if (t + 1 < 8) {
                    A = acc ? c1 : c0;
                    if (t + 2 < 8) {
                        c0 = wS[st.E + d.dDel[t + 2]];
                        c1 = wS[st.E + d.dDel[t + 1] + d.dDel[t + 2]];
                    }
                }
            }
        };
#pragma unroll 1
        for (uint32_t k = 0; k < windows; k += 2) {
            chain(d0);
            chain(d1);
        }
    }
    const unsigned long long t1 = clock64();
    if ((lane & 31u) == 0) cycles[lane >> 5] = t1 - t0;
    sink[lane] = fold + (uint32_t)st.E + (uint32_t)st.EJ + lat[0] + (PART == 6 ? 0u : histS[lane]);
}

cudaError_t launch_sweep_floor(int part, uint32_t windows, unsigned long long *cycles, uint32_t *sink,
                               unsigned long long *hist_dummy, cudaStream_t s)
{
    const size_t smem = smem_weights_bytes(kModeWeight, kFloorN) + smem_hist_bytes(kModeWeight, kFloorN) +
                        (size_t)kFloorL * kFloorWPR * kFloorCpb * 4;
    auto go = [&](auto kern) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<1, kFloorCpb, smem, s>>>(windows, cycles, sink, hist_dummy);
        return cudaGetLastError();
    };
    switch (part) {
    case 0: return go(k_sweep_floor<0>);
    case 1: return go(k_sweep_floor<1>);
    case 2: return go(k_sweep_floor<2>);
    case 3: return go(k_sweep_floor<3>);
    case 4: return go(k_sweep_floor<4>);
    case 5: return go(k_sweep_floor<5>);
    default: return go(k_sweep_floor<6>);
    }
}

}  // namespace muca
