// devlogf.cu -- test infrastructure: CUDA's single-precision logf at every
// value u01fixedpt<float> can take, for the oracle's acceptance test.
//
// The reference kernels accept a proposal when
//     log(r123::u01fixedpt<float>(r1)) < diff
// (muca_delta_multigpu.cu:781,816, produce2_multigpu.cu:446,481), evaluated on the
// GPU, i.e. with CUDA's logf.  CUDA's logf and the host libm's logf differ by
// one ulp on 665,345 of the 2^23 possible u (measured on a GB300; the x86 and
// aarch64 libm agree with each other), so a CPU restatement that calls libm
// takes a different decision whenever diff falls on that ulp -- rare per
// attempt, certain over a long weight run.  This library calls CUDA's logf on
// the device for all 2^23 inputs; the oracle then looks the value up.
//
// u01fixedpt<float>(r) = (1 | (r >> 8)) * 2^-24 = (2k + 1) * 2^-24 with
// k = r >> 9, exact in float, so entry k of the table belongs to every r with
// r >> 9 == k.
#include <cuda_runtime.h>
#include <cstdio>

namespace {

constexpr unsigned kValues = 1u << 23;

__global__ void k_logf_all(float *out)
{
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < kValues) out[k] = logf((float)(2u * k + 1u) * 5.9604644775390625e-8f);
}

}  // namespace

// out: host array of 2^23 floats.  Returns 0, or -1 with a message in err.
extern "C" int orc_device_logf_table(int device, float *out, char *err, int errlen)
{
    float *d = nullptr;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaMalloc(&d, sizeof(float) * kValues);
    if (e == cudaSuccess) {
        k_logf_all<<<kValues / 256, 256>>>(d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d, sizeof(float) * kValues, cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (e != cudaSuccess) {
        std::snprintf(err, (size_t)errlen, "%s", cudaGetErrorString(e));
        return -1;
    }
    return 0;
}
