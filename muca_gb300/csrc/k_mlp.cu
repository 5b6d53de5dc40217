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
//   forward  per tile of 32 points: the layer matrix staged (transposed) in
//            shared memory, the activations kept transposed [unit][point],
//            and each of 256 threads accumulates a 4 x 4 register tile
//            (4 units x 4 points: two 16-byte shared loads per 16 FMAs);
//            pre-activations kept;
//   backward per tile: dL/dz of every layer, the W^T products in the same
//            4 x 4 register tiles;
//   wgrad    per layer, dW = dZ^T H and db = sum dZ, 32 x 32 output tiles
//            with the minibatch split over kWSplit slices (blocks), then the
//            slices summed in a fixed order (no atomics: deterministic);
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
constexpr int kPitch = kHid + 4;  // row pitch of a staged layer matrix: 16-byte rows
constexpr int kWSplit = 16;    // minibatch slices of the weight gradients
static_assert(kThreads == 8 * 32 && kTile == 4 * 8 && kHid == 4 * 32, "4 x 4 register tiles");

size_t mlp_param_count() { return kParams; }

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
__device__ __forceinline__ float dsilu(float z)
{
    const float s = sigm(z);
    return s * (1.0f + z * (1.0f - s));
}

// Stage W [kHid][kHid] (16-byte aligned) transposed into sW[j][o] (row pitch kPitch).
__device__ __forceinline__ void stage_transposed(const float *__restrict__ W, float *sW)
{
    for (int t = threadIdx.x; t < kHid * kHid / 4; t += blockDim.x) {
        const int o = (4 * t) / kHid, j = 4 * t - o * kHid;
        const float4 v = reinterpret_cast<const float4 *>(W)[t];
        sW[(j + 0) * kPitch + o] = v.x;
        sW[(j + 1) * kPitch + o] = v.y;
        sW[(j + 2) * kPitch + o] = v.z;
        sW[(j + 3) * kPitch + o] = v.w;
    }
}
// Stage W [kHid][kHid] as is into sW[o][j] (row pitch kPitch).
__device__ __forceinline__ void stage_plain(const float *__restrict__ W, float *sW)
{
    for (int t = threadIdx.x; t < kHid * kHid / 4; t += blockDim.x) {
        const int o = (4 * t) / kHid, j = 4 * t - o * kHid;
        *reinterpret_cast<float4 *>(sW + o * kPitch + j) = reinterpret_cast<const float4 *>(W)[t];
    }
}

// acc[a][b] += sum over k < kHid of A[k][a0 + a] * Bt[k][b0 + b]: A rows of
// pitch kPitch, Bt rows of kTile (both shared memory, 16-byte aligned), in k
// order.  The lanes of a warp share b0 (a broadcast load) and take 32
// consecutive a0 (one 512-byte row segment).
__device__ __forceinline__ void tile_product(const float *__restrict__ A, const float *__restrict__ Bt, int a0,
                                             int b0, float (&acc)[4][4])
{
#pragma unroll 4
    for (int k = 0; k < kHid; ++k) {
        const float4 a = *reinterpret_cast<const float4 *>(A + k * kPitch + a0);
        const float4 b = *reinterpret_cast<const float4 *>(Bt + k * kTile + b0);
        const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
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
// Y gets the outputs.  Thread (ty, tx) = (threadIdx.x / 32, threadIdx.x % 32)
// owns units 4 tx .. 4 tx + 3 of points 4 ty .. 4 ty + 3 of the tile.
__global__ void __launch_bounds__(kThreads) k_mlp_forward(const float *__restrict__ P, const float *__restrict__ Xb,
                                                          uint32_t B, float *__restrict__ Z, float *__restrict__ Y)
{
    extern __shared__ __align__(16) float sm[];
    float *sW = sm;                      // [kHid][kPitch]
    float *hA = sW + kHid * kPitch;      // [kHid][kTile], activations transposed
    float *hB = hA + kHid * kTile;       // [kHid][kTile]
    float *sx = hB + kHid * kTile;       // [kTile][kIn]
    __shared__ float red[kThreads / 32][kTile];
    const uint32_t p0 = blockIdx.x * kTile;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int a0 = 4 * tx, b0 = 4 * ty;
    for (int t = threadIdx.x; t < kTile * kIn; t += blockDim.x) {
        const uint32_t p = p0 + t / kIn;
        sx[t] = p < B ? Xb[(size_t)p0 * kIn + t] : 0.0f;
    }
    __syncthreads();
    // layer 1 (4 inputs): straight from global
    {
        float z[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            float w[kIn];
#pragma unroll
            for (int i = 0; i < kIn; ++i) w[i] = P[kOffW1 + (a0 + a) * kIn + i];
            const float b = P[kOffB1 + a0 + a];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float v = b;
#pragma unroll
                for (int i = 0; i < kIn; ++i) v = fmaf(w[i], sx[(b0 + q) * kIn + i], v);
                z[a][q] = v;
            }
            *reinterpret_cast<float4 *>(hA + (a0 + a) * kTile + b0) =
                make_float4(silu(z[a][0]), silu(z[a][1]), silu(z[a][2]), silu(z[a][3]));
        }
        if (Z)
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (p0 + b0 + q < B)
                    *reinterpret_cast<float4 *>(Z + (size_t)(p0 + b0 + q) * kHid + a0) =
                        make_float4(z[0][q], z[1][q], z[2][q], z[3][q]);
    }
    // layers 2 and 3
    float *hin = hA, *hout = hB;
    for (int l = 0; l < 2; ++l) {
        const float *W = P + (l == 0 ? kOffW2 : kOffW3);
        const float *bias = P + (l == 0 ? kOffB2 : kOffB3);
        __syncthreads();  // previous readers of sW are done; hin is written
        stage_transposed(W, sW);
        __syncthreads();
        float acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const float b = bias[a0 + a];
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[a][q] = b;
        }
        tile_product(sW, hin, a0, b0, acc);
#pragma unroll
        for (int a = 0; a < 4; ++a)
            *reinterpret_cast<float4 *>(hout + (a0 + a) * kTile + b0) =
                make_float4(silu(acc[a][0]), silu(acc[a][1]), silu(acc[a][2]), silu(acc[a][3]));
        if (Z)
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (p0 + b0 + q < B)
                    *reinterpret_cast<float4 *>(Z + ((size_t)(l + 1) * B + p0 + b0 + q) * kHid + a0) =
                        make_float4(acc[0][q], acc[1][q], acc[2][q], acc[3][q]);
        float *t = hin;
        hin = hout;
        hout = t;
    }
    __syncthreads();
    // output layer: point tx, units 16 ty .. 16 ty + 15, then the 8 partial
    // sums in a fixed order
    {
        float s = 0.0f;
#pragma unroll
        for (int j = 16 * ty; j < 16 * ty + 16; ++j) s = fmaf(P[kOffW4 + j], hin[j * kTile + tx], s);
        red[ty][tx] = s;
    }
    __syncthreads();
    if (ty == 0 && p0 + tx < B) {
        float s = P[kOffB4];
#pragma unroll
        for (int g = 0; g < kThreads / 32; ++g) s += red[g][tx];
        Y[p0 + tx] = s;
    }
}

// Backward over B points: dy = 2 (y - t) / B (the gradient of the mean
// squared error), then dL/dz of layers 3, 2, 1 into dZ [3][B][kHid] (layer
// l - 1 at offset l - 1) and dy into dZ + 3 B kHid; the block's sum of
// squared errors into lpart[blockIdx.x].  Register tiles as in the forward
// pass: thread (ty, tx) owns units 4 tx .. 4 tx + 3 of points 4 ty .. 4 ty + 3.
__global__ void __launch_bounds__(kThreads) k_mlp_backward(const float *__restrict__ P, const float *__restrict__ Tb,
                                                           const float *__restrict__ Y, const float *__restrict__ Z,
                                                           uint32_t B, float *__restrict__ dZ,
                                                           float *__restrict__ lpart)
{
    extern __shared__ __align__(16) float sm[];
    float *sW = sm;                      // [kHid][kPitch], W as is: sW[o][j]
    float *dA = sW + kHid * kPitch;      // [kHid][kTile], deltas transposed
    float *dB = dA + kHid * kTile;       // [kHid][kTile]
    float *sdy = dB + kHid * kTile;      // [kTile]
    __shared__ float red[kThreads / 32];
    const uint32_t p0 = blockIdx.x * kTile;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int a0 = 4 * tx, b0 = 4 * ty;
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
        float v[4][4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t p = p0 + b0 + q;
            float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (p < B) z = *reinterpret_cast<const float4 *>(Z + ((size_t)2 * B + p) * kHid + a0);
            const float zz[4] = {z.x, z.y, z.z, z.w};
#pragma unroll
            for (int a = 0; a < 4; ++a) v[a][q] = p < B ? sdy[b0 + q] * P[kOffW4 + a0 + a] * dsilu(zz[a]) : 0.0f;
            if (p < B)
                *reinterpret_cast<float4 *>(dZ + ((size_t)2 * B + p) * kHid + a0) =
                    make_float4(v[0][q], v[1][q], v[2][q], v[3][q]);
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
            *reinterpret_cast<float4 *>(dA + (a0 + a) * kTile + b0) = make_float4(v[a][0], v[a][1], v[a][2], v[a][3]);
    }
    // dz2 = (W3^T dz3) * silu'(z2), dz1 = (W2^T dz2) * silu'(z1): this
    // thread's units are now the inputs j = a0 .. a0 + 3 of layer l + 1
    float *din = dA, *dout = dB;
    for (int l = 2; l >= 1; --l) {
        const float *W = P + (l == 2 ? kOffW3 : kOffW2);
        __syncthreads();
        stage_plain(W, sW);
        __syncthreads();
        float acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[a][q] = 0.0f;
        tile_product(sW, din, a0, b0, acc);
        float v[4][4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t p = p0 + b0 + q;
            float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (p < B) z = *reinterpret_cast<const float4 *>(Z + ((size_t)(l - 1) * B + p) * kHid + a0);
            const float zz[4] = {z.x, z.y, z.z, z.w};
#pragma unroll
            for (int a = 0; a < 4; ++a) v[a][q] = p < B ? acc[a][q] * dsilu(zz[a]) : 0.0f;
            if (p < B)
                *reinterpret_cast<float4 *>(dZ + ((size_t)(l - 1) * B + p) * kHid + a0) =
                    make_float4(v[0][q], v[1][q], v[2][q], v[3][q]);
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
            *reinterpret_cast<float4 *>(dout + (a0 + a) * kTile + b0) =
                make_float4(v[a][0], v[a][1], v[a][2], v[a][3]);
        float *t = din;
        din = dout;
        dout = t;
    }
}

// Weight gradient of one layer, one slice of the minibatch (blockIdx.z of
// kWSplit): part[z][o][i] = sum over the slice's points p of D[p][o] H[p][i],
// i <= in_dim, with H[p][in_dim] taken as 1 (the bias column).  H is Xb
// (hsilu = 0) or silu of the previous layer's pre-activations (hsilu = 1).
// 32 x 32 output tiles, 256 threads x 4 outputs, the slice in chunks of 32
// points.
__global__ void __launch_bounds__(256) k_mlp_wgrad(const float *__restrict__ D, const float *__restrict__ H,
                                                   uint32_t B, int out_dim, int in_dim, int hsilu,
                                                   float *__restrict__ part)
{
    __shared__ float sD[32][33], sH[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i0 = blockIdx.x * 32, o0 = blockIdx.y * 32;
    const uint32_t slice = (B + kWSplit - 1) / kWSplit;
    const uint32_t c0 = blockIdx.z * slice, c1 = min(B, c0 + slice);
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (uint32_t c = c0; c < c1; c += 32) {
        for (int t = threadIdx.x; t < 32 * 32; t += 256) {
            const int r = t >> 5, q = t & 31;
            const uint32_t p = c + r;
            const int oo = o0 + q, ii = i0 + q;
            sD[r][q] = (p < c1 && oo < out_dim) ? D[(size_t)p * out_dim + oo] : 0.0f;
            float h = 0.0f;
            if (p < c1) {
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
        if (oo < out_dim && i <= in_dim) part[((size_t)blockIdx.z * out_dim + oo) * (in_dim + 1) + i] = acc[k];
    }
}

// The slices' partial gradients summed in slice order: gW[o][i] (i < in_dim)
// and gb[o] (i = in_dim).
__global__ void k_mlp_wsum(const float *__restrict__ part, int out_dim, int in_dim, float *__restrict__ gW,
                           float *__restrict__ gb)
{
    const int n = out_dim * (in_dim + 1);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        float s = 0.0f;
#pragma unroll
        for (int z = 0; z < kWSplit; ++z) s += part[(size_t)z * n + t];
        const int o = t / (in_dim + 1), i = t - o * (in_dim + 1);
        if (i < in_dim) gW[(size_t)o * in_dim + i] = s;
        else gb[o] = s;
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

static size_t fwd_smem() { return sizeof(float) * ((size_t)kHid * kPitch + 2 * kTile * kHid + kTile * kIn); }
static size_t bwd_smem() { return sizeof(float) * ((size_t)kHid * kPitch + 2 * kTile * kHid + kTile); }

cudaError_t mlp_prepare()
{
    cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwd_smem());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bwd_smem());
    return e;
}

// Scratch of a minibatch of B points, in floats from the (16-byte aligned)
// base: Xb [B][kIn] at 0, Tb [B] at 4B, Y [B] at 5B, then 16-byte aligned
// Z [3][B][kHid] (the kernels store 4 units at once), dZ [3][B][kHid] + dy [B],
// the loss partials, and 16-byte aligned the weight gradients' slice partials.
struct MlpScratch {
    float *Xb, *Tb, *Y, *Z, *dZ, *lpart, *wpart;
    size_t floats;
};
static size_t align4f(size_t n) { return (n + 3) / 4 * 4; }
static MlpScratch mlp_scratch_layout(float *base, uint32_t B)
{
    MlpScratch m;
    const size_t z = align4f((size_t)B * kIn + 2ull * B);
    const size_t dz = z + 3ull * B * kHid;
    const size_t lp = dz + 3ull * B * kHid + B;
    const size_t wp = align4f(lp + (B + kTile - 1) / kTile);
    m.Xb = base;
    m.Tb = base ? base + (size_t)B * kIn : nullptr;
    m.Y = base ? base + (size_t)B * kIn + B : nullptr;
    m.Z = base ? base + z : nullptr;
    m.dZ = base ? base + dz : nullptr;
    m.lpart = base ? base + lp : nullptr;
    m.wpart = base ? base + wp : nullptr;
    m.floats = wp + (size_t)kWSplit * kHid * (kHid + 1);
    return m;
}

size_t mlp_scratch_floats(uint32_t B) { return mlp_scratch_layout(nullptr, B).floats; }

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
    const MlpScratch sc = mlp_scratch_layout(scratch, B);
    float *Xb = sc.Xb, *Tb = sc.Tb, *Y = sc.Y, *Z = sc.Z, *dZ = sc.dZ, *lpart = sc.lpart, *wpart = sc.wpart;
    const int nt = (int)((B + kTile - 1) / kTile);
    if (gather) {
        k_mlp_gather<<<(B + 255) / 256, 256, 0, s>>>(X, T, n, B, step, seed, Xb, Tb);
    }
    k_mlp_forward<<<nt, kThreads, fwd_smem(), s>>>(P, Xb, B, Z, Y);
    k_mlp_backward<<<nt, kThreads, bwd_smem(), s>>>(P, Tb, Y, Z, B, dZ, lpart);
    // per layer: slices of the minibatch, then their sum in slice order (one
    // scratch of partials serves the layers one after the other)
    const dim3 g1(1, kHid / 32, kWSplit), gh((kHid + 1 + 31) / 32, kHid / 32, kWSplit),
        g4((kHid + 1 + 31) / 32, 1, kWSplit);
    k_mlp_wgrad<<<g1, 256, 0, s>>>(dZ, Xb, B, kHid, kIn, 0, wpart);
    k_mlp_wsum<<<(kHid * (kIn + 1) + 255) / 256, 256, 0, s>>>(wpart, kHid, kIn, G + kOffW1, G + kOffB1);
    k_mlp_wgrad<<<gh, 256, 0, s>>>(dZ + (size_t)B * kHid, Z, B, kHid, kHid, 1, wpart);
    k_mlp_wsum<<<(kHid * (kHid + 1) + 255) / 256, 256, 0, s>>>(wpart, kHid, kHid, G + kOffW2, G + kOffB2);
    k_mlp_wgrad<<<gh, 256, 0, s>>>(dZ + 2ull * B * kHid, Z + (size_t)B * kHid, B, kHid, kHid, 1, wpart);
    k_mlp_wsum<<<(kHid * (kHid + 1) + 255) / 256, 256, 0, s>>>(wpart, kHid, kHid, G + kOffW3, G + kOffB3);
    k_mlp_wgrad<<<g4, 256, 0, s>>>(dZ + 3ull * B * kHid, Z + 2ull * B * kHid, B, 1, kHid, 1, wpart);
    k_mlp_wsum<<<1, 256, 0, s>>>(wpart, 1, kHid, G + kOffW4, G + kOffB4);
    if (m && v) k_mlp_adam<<<(kParams + 255) / 256, 256, 0, s>>>(P, G, m, v, step, lr);
    k_mlp_finish<<<1, 32, 0, s>>>(lpart, nt, B, losses, losses_cap, step, base);
    return cudaGetLastError();
}

}  // namespace muca
