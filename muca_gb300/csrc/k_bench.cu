// k_bench.cu -- measurement kernel for the integer-pipe roofline.
//
// The sweep kernels spend most of their issue slots on Philox4x32 blocks
// (two per four Metropolis attempts).  k_philox_peak generates Philox blocks
// in exactly the form the sweeps use them (per-thread key, counter words 1..3
// fixed, word 0 counting) at full occupancy with nothing else to do, so its
// rate is the ceiling of "Philox blocks per second" on this GPU.
#include "muca_device.cuh"
#include "muca_internal.h"

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

}  // namespace muca
