// k_mlp.cu -- the learned warm start: a small MLP trained and evaluated by
// hand-written FP32 kernels.
//
// The network maps (L/128, T, Delta, x) to y, where x = E_Delta/N is the
// position on the weight axis and y = (lnW(E_Delta) - mean lnW) / N is the
// log weight per site with its mean removed (lnW is extensive in N, so the
// per-site form is what transfers between lattice sizes).  Three hidden
// layers of 128 SiLU units, one linear output; parameters and arithmetic are
// FP32.  It replaces the trivial (zero) or extrapolated initial weight of the
// reference's `continuing` path (muca_delta_multigpu.cu:223-235); the weight
// recursion then runs to the same flatness criterion.
//
// Parameters live in one flat array, each layer's matrix row-major [out][in]
// followed by its bias (offsets kOff*).  A training step is
//   gather   minibatch indices from Philox(step, k), inputs and targets;
//   forward  per tile of 32 points: the layer matrix staged transposed in
//            shared memory, 256 threads x 16 outputs, pre-activations kept;
//   backward per tile: dL/dz of every layer (W^T products from shared memory);
//   wgrad    per layer, dW = dZ^T H and db = sum dZ, a 32x32-tiled product
//            over the minibatch in a fixed order (no atomics: deterministic);
//   adam     elementwise, bias-corrected, step count on the device.
// The step reads its step number from device memory, so a CUDA graph of K
// steps can be replayed.
#include "muca_device.cuh"
#include "muca_internal.h"

namespace muca {

constexpr int kIn = 4, kHid = 128;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kHid * kIn;
constexpr int kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid * kHid;
constexpr int kOffW4 = kOffB3 + kHid, kOffB4 = kOffW4 + kHid;
constexpr int kParams = kOffB4 + 1;
static_assert(kParams == 33793, "parameter layout");
constexpr int kTile = 32;      // points per block in forward/backward
constexpr int kThreads = 256;  // threads per block in forward/backward

size_t mlp_param_count() { return kParams; }

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
__device__ __forceinline__ float dsilu(float z)
{
    const float s = sigm(z);
    return s * (1.0f + z * (1.0f - s));
}

// Stage W [kHid][kHid] transposed into sW[j][o] (row pitch kHid + 1).
__device__ __forceinline__ void stage_transposed(const float *__restrict__ W, float *sW)
{
    for (int t = threadIdx.x; t < kHid * kHid; t += blockDim.x) {
        const int o = t / kHid, j = t - o * kHid;
        sW[j * (kHid + 1) + o] = W[t];
    }
}
// Stage W [kHid][kHid] as is into sW[o][j] (row pitch kHid + 1).
__device__ __forceinline__ void stage_plain(const float *__restrict__ W, float *sW)
{
    for (int t = threadIdx.x; t < kHid * kHid; t += blockDim.x) {
        const int o = t / kHid, j = t - o * kHid;
        sW[o * (kHid + 1) + j] = W[t];
    }
}

// Minibatch gather: point k of step s is index Philox(k, s) mod n (all of
// them, in order, when the batch is the whole set: n == B and s == ~0u).
__global__ void k_mlp_gather(const float *__restrict__ X, const float *__restrict__ T, uint32_t n, uint32_t B,
                             const uint32_t *__restrict__ step, uint32_t seed, float *__restrict__ Xb,
                             float *__restrict__ Tb)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= B) return;
    uint32_t idx = k;
    if (step) {
        RoundKeys<10> key;
        key.init(seed, 0x4d4c5000u);
        const uint4 r = philox<10>(k, *step, 0x57A27u, 0u, key);
        idx = (uint32_t)(((unsigned long long)r.x * n) >> 32);
    }
#pragma unroll
    for (int i = 0; i < kIn; ++i) Xb[(size_t)k * kIn + i] = X[(size_t)idx * kIn + i];
    if (Tb) Tb[k] = T ? T[idx] : 0.0f;
}

// Forward over B points.  Z (optional) gets the pre-activations [3][B][kHid];
// Y gets the outputs.
__global__ void __launch_bounds__(kThreads) k_mlp_forward(const float *__restrict__ P, const float *__restrict__ Xb,
                                                          uint32_t B, float *__restrict__ Z, float *__restrict__ Y)
{
    extern __shared__ __align__(16) float sm[];
    float *sW = sm;                                  // [kHid][kHid + 1]
    float *hA = sW + kHid * (kHid + 1);              // [kTile][kHid]
    float *hB = hA + kTile * kHid;                   // [kTile][kHid]
    float *sx = hB + kTile * kHid;                   // [kTile][kIn]
    const uint32_t p0 = blockIdx.x * kTile;
    const int o = threadIdx.x % kHid, pg = threadIdx.x / kHid;  // pg in {0, 1}
    constexpr int kPer = kTile / (kThreads / kHid);             // 16 points per thread
    for (int t = threadIdx.x; t < kTile * kIn; t += blockDim.x) {
        const uint32_t p = p0 + t / kIn;
        sx[t] = p < B ? Xb[(size_t)p0 * kIn + t] : 0.0f;
    }
    __syncthreads();
    // layer 1 (4 inputs): straight from global
    {
        float w[kIn];
#pragma unroll
        for (int i = 0; i < kIn; ++i) w[i] = P[kOffW1 + o * kIn + i];
        const float b = P[kOffB1 + o];
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const int p = pg + 2 * k;
            float z = b;
#pragma unroll
            for (int i = 0; i < kIn; ++i) z = fmaf(w[i], sx[p * kIn + i], z);
            if (Z && p0 + p < B) Z[(size_t)(p0 + p) * kHid + o] = z;
            hA[p * kHid + o] = silu(z);
        }
    }
    // layers 2 and 3
    float *hin = hA, *hout = hB;
    for (int l = 0; l < 2; ++l) {
        const float *W = P + (l == 0 ? kOffW2 : kOffW3);
        const float b = P[(l == 0 ? kOffB2 : kOffB3) + o];
        __syncthreads();  // previous readers of sW are done
        stage_transposed(W, sW);
        __syncthreads();
        float acc[kPer];
#pragma unroll
        for (int k = 0; k < kPer; ++k) acc[k] = b;
        for (int j = 0; j < kHid; ++j) {
            const float w = sW[j * (kHid + 1) + o];
#pragma unroll
            for (int k = 0; k < kPer; ++k) acc[k] = fmaf(w, hin[(pg + 2 * k) * kHid + j], acc[k]);
        }
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const int p = pg + 2 * k;
            if (Z && p0 + p < B) Z[((size_t)(l + 1) * B + p0 + p) * kHid + o] = acc[k];
            hout[p * kHid + o] = silu(acc[k]);
        }
        float *t = hin;
        hin = hout;
        hout = t;
    }
    __syncthreads();
    // output layer: one warp per point group, reduced over the 128 inputs
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int p = warp; p < kTile; p += kThreads / 32) {
        float s = 0.0f;
        for (int j = lane; j < kHid; j += 32) s = fmaf(P[kOffW4 + j], hin[p * kHid + j], s);
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
        if (lane == 0 && p0 + p < B) Y[p0 + p] = s + P[kOffB4];
    }
}

// Backward over B points: dy = 2 (y - t) / B (the gradient of the mean
// squared error), then dL/dz of layers 3, 2, 1 into dZ [3][B][kHid] (layer
// l - 1 at offset l - 1) and dy into dZ + 3 B kHid; the block's sum of
// squared errors into lpart[blockIdx.x].
__global__ void __launch_bounds__(kThreads) k_mlp_backward(const float *__restrict__ P, const float *__restrict__ Tb,
                                                           const float *__restrict__ Y, const float *__restrict__ Z,
                                                           uint32_t B, float *__restrict__ dZ,
                                                           float *__restrict__ lpart)
{
    extern __shared__ __align__(16) float sm[];
    float *sW = sm;                      // [kHid][kHid + 1], W as is: sW[o][j]
    float *dA = sW + kHid * (kHid + 1);  // [kTile][kHid]
    float *dB = dA + kTile * kHid;       // [kTile][kHid]
    float *sdy = dB + kTile * kHid;      // [kTile]
    __shared__ float red[kThreads / 32];
    const uint32_t p0 = blockIdx.x * kTile;
    const int o = threadIdx.x % kHid, pg = threadIdx.x / kHid;
    constexpr int kPer = kTile / (kThreads / kHid);
    float sq = 0.0f;
    if (threadIdx.x < kTile) {
        const uint32_t p = p0 + threadIdx.x;
        float d = 0.0f;
        if (p < B) {
            const float e = Y[p] - Tb[p];
            sq = e * e;
            d = 2.0f * e / (float)B;
            dZ[(size_t)3 * B * kHid + p] = d;
        }
        sdy[threadIdx.x] = d;
    }
    // block sum of squared errors (fixed order)
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int w = 0; w < kThreads / 32; ++w) s += red[w];
        lpart[blockIdx.x] = s;
    }
    // layer 3 output: dz3 = dy * W4[o] * silu'(z3)
    {
        const float w4 = P[kOffW4 + o];
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const int p = pg + 2 * k;
            float v = 0.0f;
            if (p0 + p < B) {
                v = sdy[p] * w4 * dsilu(Z[((size_t)2 * B + p0 + p) * kHid + o]);
                dZ[((size_t)2 * B + p0 + p) * kHid + o] = v;
            }
            dA[p * kHid + o] = v;
        }
    }
    // dz2 = (W3^T dz3) * silu'(z2), dz1 = (W2^T dz2) * silu'(z1)
    float *din = dA, *dout = dB;
    for (int l = 2; l >= 1; --l) {
        const float *W = P + (l == 2 ? kOffW3 : kOffW2);
        __syncthreads();
        stage_plain(W, sW);
        __syncthreads();
        float acc[kPer];
#pragma unroll
        for (int k = 0; k < kPer; ++k) acc[k] = 0.0f;
        const int j = o;  // this thread's input unit of layer l+1
        for (int oo = 0; oo < kHid; ++oo) {
            const float w = sW[oo * (kHid + 1) + j];
#pragma unroll
            for (int k = 0; k < kPer; ++k) acc[k] = fmaf(w, din[(pg + 2 * k) * kHid + oo], acc[k]);
        }
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const int p = pg + 2 * k;
            float v = 0.0f;
            if (p0 + p < B) {
                v = acc[k] * dsilu(Z[((size_t)(l - 1) * B + p0 + p) * kHid + j]);
                dZ[((size_t)(l - 1) * B + p0 + p) * kHid + j] = v;
            }
            dout[p * kHid + j] = v;
        }
        float *t = din;
        din = dout;
        dout = t;
    }
}

// Weight gradient of one layer: gW[o][i] = sum_p D[p][o] H[p][i] and
// gb[o] = sum_p D[p][o], H[p][in_dim] taken as 1.  H is Xb (hsilu = 0) or
// silu of the previous layer's pre-activations (hsilu = 1).  32 x 32 output
// tiles, 256 threads x 4 outputs, the minibatch in chunks of 32 points.
__global__ void __launch_bounds__(256) k_mlp_wgrad(const float *__restrict__ D, const float *__restrict__ H,
                                                   uint32_t B, int out_dim, int in_dim, int hsilu,
                                                   float *__restrict__ gW, float *__restrict__ gb)
{
    __shared__ float sD[32][33], sH[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i0 = blockIdx.x * 32, o0 = blockIdx.y * 32;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (uint32_t c = 0; c < B; c += 32) {
        for (int t = threadIdx.x; t < 32 * 32; t += 256) {
            const int r = t >> 5, q = t & 31;
            const uint32_t p = c + r;
            const int oo = o0 + q, ii = i0 + q;
            sD[r][q] = (p < B && oo < out_dim) ? D[(size_t)p * out_dim + oo] : 0.0f;
            float h = 0.0f;
            if (p < B) {
                if (ii < in_dim) {
                    const float v = H[(size_t)p * in_dim + ii];
                    h = hsilu ? silu(v) : v;
                } else if (ii == in_dim) {
                    h = 1.0f;
                }
            }
            sH[r][q] = h;
        }
        __syncthreads();
#pragma unroll 8
        for (int r = 0; r < 32; ++r) {
            const float h = sH[r][tx];
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[k] = fmaf(sD[r][ty + 8 * k], h, acc[k]);
        }
        __syncthreads();
    }
    const int i = i0 + tx;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int oo = o0 + ty + 8 * k;
        if (oo >= out_dim) continue;
        if (i < in_dim) gW[(size_t)oo * in_dim + i] = acc[k];
        else if (i == in_dim) gb[oo] = acc[k];
    }
}

// Adam (Kingma & Ba, 2015, Algorithm 1) with bias correction; t = *step + 1.
__global__ void k_mlp_adam(float *__restrict__ P, const float *__restrict__ G, float *__restrict__ m,
                           float *__restrict__ v, const uint32_t *__restrict__ step, float lr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float t = (float)(*step + 1u);
    const float g = G[i];
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.0f - powf(b1, t));
    const float vh = vi / (1.0f - powf(b2, t));
    P[i] -= lr * mh / (sqrtf(vh) + eps);
}

// Loss of the step (sum of the block partials in order, / B) into
// losses[*step] when losses is given, then the step count advances.
// losses[*step - *base] when step is given, else losses[0] (a gradient
// evaluation without a step).
__global__ void k_mlp_finish(const float *__restrict__ lpart, int nblocks, uint32_t B, float *__restrict__ losses,
                             uint32_t losses_cap, uint32_t *__restrict__ step, const uint32_t *__restrict__ base)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float s = 0.0f;
    for (int b = 0; b < nblocks; ++b) s += lpart[b];
    if (!step) {
        if (losses && losses_cap) losses[0] = s / (float)B;
        return;
    }
    const uint32_t t = *step, k = t - (base ? *base : 0u);
    if (losses && k < losses_cap) losses[k] = s / (float)B;
    *step = t + 1u;
}

static size_t fwd_smem() { return sizeof(float) * ((size_t)kHid * (kHid + 1) + 2 * kTile * kHid + kTile * kIn); }
static size_t bwd_smem() { return sizeof(float) * ((size_t)kHid * (kHid + 1) + 2 * kTile * kHid + kTile); }

cudaError_t mlp_prepare()
{
    cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwd_smem());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bwd_smem());
    return e;
}

size_t mlp_scratch_floats(uint32_t B)
{
    // Xb, Tb, Y, Z (3 layers), dZ (3 layers + dy), lpart
    return (size_t)B * kIn + B + B + 3ull * B * kHid + (3ull * B * kHid + B) + (B + kTile - 1) / kTile;
}

cudaError_t launch_mlp_forward(const float *P, const float *Xb, uint32_t B, float *Z, float *Y, cudaStream_t s)
{
    if (B == 0) return cudaSuccess;
    k_mlp_forward<<<(B + kTile - 1) / kTile, kThreads, fwd_smem(), s>>>(P, Xb, B, Z, Y);
    return cudaGetLastError();
}

// One gradient evaluation (and, with m/v, one Adam step) on the minibatch
// in scratch; gather == true draws it from (X, T, n) first.
cudaError_t launch_mlp_step(float *P, float *G, float *m, float *v, const float *X, const float *T, uint32_t n,
                            uint32_t B, uint32_t *step, const uint32_t *base, uint32_t seed, bool gather, float lr,
                            float *scratch, float *losses, uint32_t losses_cap, cudaStream_t s)
{
    float *Xb = scratch, *Tb = Xb + (size_t)B * kIn, *Y = Tb + B, *Z = Y + B;
    float *dZ = Z + 3ull * B * kHid, *lpart = dZ + 3ull * B * kHid + B;
    const int nt = (int)((B + kTile - 1) / kTile);
    if (gather) {
        k_mlp_gather<<<(B + 255) / 256, 256, 0, s>>>(X, T, n, B, step, seed, Xb, Tb);
    }
    k_mlp_forward<<<nt, kThreads, fwd_smem(), s>>>(P, Xb, B, Z, Y);
    k_mlp_backward<<<nt, kThreads, bwd_smem(), s>>>(P, Tb, Y, Z, B, dZ, lpart);
    const dim3 g1(1, kHid / 32), gh((kHid + 1 + 31) / 32, kHid / 32), g4((kHid + 1 + 31) / 32, 1);
    k_mlp_wgrad<<<g1, 256, 0, s>>>(dZ, Xb, B, kHid, kIn, 0, G + kOffW1, G + kOffB1);
    k_mlp_wgrad<<<gh, 256, 0, s>>>(dZ + (size_t)B * kHid, Z, B, kHid, kHid, 1, G + kOffW2, G + kOffB2);
    k_mlp_wgrad<<<gh, 256, 0, s>>>(dZ + 2ull * B * kHid, Z + (size_t)B * kHid, B, kHid, kHid, 1, G + kOffW3,
                                   G + kOffB3);
    k_mlp_wgrad<<<g4, 256, 0, s>>>(dZ + 3ull * B * kHid, Z + 2ull * B * kHid, B, 1, kHid, 1, G + kOffW4, G + kOffB4);
    if (m && v) k_mlp_adam<<<(kParams + 255) / 256, 256, 0, s>>>(P, G, m, v, step, lr);
    k_mlp_finish<<<1, 32, 0, s>>>(lpart, nt, B, losses, losses_cap, step, base);
    return cudaGetLastError();
}

}  // namespace muca
