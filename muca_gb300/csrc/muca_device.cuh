// muca_device.cuh -- device primitives shared by the GB300 kernels.
//
// Philox4x32-R (Salmon et al., SC'11, sec. 3.2) with the constants of
// Random123 philox.h:232-250 and the round/key-bump order of :284-320, and the
// u01fixedpt<float> conversion of Random123 examples/uniform.hpp:195-205.
// Both are written here from the published algorithm; bit-exactness is
// checked against Random123's known-answer vectors (kat_vectors:24-29).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace muca {

constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;
constexpr uint32_t kCtrTag = 0xBADC0DEDu;  // ctr.v[3] of the sweep kernels

// Round keys: round r uses key + r * (W0, W1) (the key is bumped before every
// round except the first).
template <int R>
struct RoundKeys {
    uint32_t a[R], b[R];
    __device__ __forceinline__ void init(uint32_t k0, uint32_t k1)
    {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            a[r] = k0 + (uint32_t)r * kPhiloxW0;
            b[r] = k1 + (uint32_t)r * kPhiloxW1;
        }
    }
};

template <int R>
__device__ __forceinline__ uint4 philox(uint32_t x0, uint32_t x1, uint32_t x2, uint32_t x3, const RoundKeys<R> &k)
{
#pragma unroll
    for (int r = 0; r < R; ++r) {
        // one 32x32 -> 64-bit product per multiplier (hi and lo of mulhilo)
        const unsigned long long p0 = (unsigned long long)kPhiloxM0 * x0;
        const unsigned long long p1 = (unsigned long long)kPhiloxM1 * x2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        x0 = hi1 ^ x1 ^ k.a[r];
        x1 = lo1;
        x2 = hi0 ^ x3 ^ k.b[r];
        x3 = lo0;
    }
    return make_uint4(x0, x1, x2, x3);
}

__device__ __forceinline__ uint32_t pick(const uint4 &v, int i)
{
    return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// u01fixedpt<float>(r) = (1 | (r >> 8)) * 2^-24 = (2k + 1) 2^-24 with
// k = r >> 9 < 2^23, exact in FP32.  Formed without an int-to-float
// conversion: the float with exponent 0 and mantissa k is 1 + k 2^-23, and
// subtracting 1 - 2^-24 leaves (2k + 1) 2^-24, which has 24 significant bits
// and is therefore the exact (and so the correctly rounded) difference.
// Checked against the conversion form for all 2^23 values of k.
__device__ __forceinline__ float u01f(uint32_t r)
{
    return __fsub_rn(__uint_as_float(0x3F800000u | (r >> 9)), __uint_as_float(0x3F7FFFFFu));
}

// (float)k for a small integer k (|k| < 2^22) without an int-to-float
// conversion: 1.5 * 2^23 + k is exact in FP32 (its ulp is 1), and so is the
// difference with 1.5 * 2^23.
__device__ __forceinline__ float small_int_to_float(int k)
{
    return __fsub_rn(__int_as_float(0x4B400000 + k), 12582912.0f);
}

// Initial spin (u < 1/3.0) + (u < 2/3.0) - 1 with the float u compared in
// double (muca_delta_multigpu.cu:350).  u = k 2^-24 with k = 1 | (r >> 8) is
// exact in double, and 2^24 times the doubles nearest 1/3 and 2/3 lie
// strictly inside (5592405, 5592406) and (11184810, 11184811), so the two
// comparisons are k <= 5592405 and k <= 11184810: integer compares in place
// of FP64, which issues slowly on this GPU.
constexpr uint32_t kInitThird = 5592405u, kInitTwoThirds = 11184810u;
__device__ __forceinline__ int init_spin(uint32_t r)
{
    const uint32_t k = 1u | (r >> 8);
    return (int)(k <= kInitThird) + (int)(k <= kInitTwoThirds) - 1;
}

// Graded initial spin of worker W of `cpd` (an extension): nonzero with
// probability (2W + 1) / (2 cpd), decided exactly in integers on the top 24
// bits of r, with the sign from bit 0, so the workers' E_Delta = sum s^2
// spread evenly over [0, N] instead of clustering at 2N/3.
__device__ __forceinline__ int graded_spin(uint32_t r, uint32_t W, uint32_t cpd)
{
    const bool nz = (unsigned long long)(r >> 8) * (2ull * cpd) < ((2ull * W + 1ull) << 24);
    return nz ? ((r & 1u) ? 1 : -1) : 0;
}

// Packed lattice: 2 bits per site holding s+1 in {0,1,2}; a row of L sites is
// stored in WPR = ceil(L/16) 32-bit words (site col at bits 2*(col%16) of
// word col/16).  Device layout [block][row*WPR + word][lane]: the 32 lanes of
// a warp touch 32 consecutive words, so every access is one 128-byte line.
__device__ __forceinline__ uint32_t spin_code(uint32_t word, uint32_t col) { return (word >> (2u * (col & 15u))) & 3u; }

constexpr uint32_t kZeroWord = 0x55555555u;  // sixteen spins of value 0

}  // namespace muca
