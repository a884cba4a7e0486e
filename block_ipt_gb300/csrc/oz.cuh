// oz.cuh - operand splitting of the FP64-accurate tensor-core product
// (internal; host and device).
//
// The product Y = Delta X with FP64 operands runs on the FP16 tensor cores
// by the error-free split-operand scheme of Ozaki, Ogita, Oishi and Rump
// ("Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applications", Numer. Algorithms
// 59 (2012)), in the fixed-point form that Mukunoki, Ozaki, Ogita and Imamura
// run on tensor cores ("DGEMM using Tensor Cores, and Its Accurate and
// Reproducible Versions", ISC 2020):
//
//  * every row i of Delta is scaled by 2^-e_i, e_i the smallest exponent
//    with max_j |Delta_ij| < 2^e_i, and rounded to the 48-bit integer
//    Q_ij = round(Delta_ij 2^(48 - e_i)); every column c of X likewise with
//    its own exponent f_c;
//  * Q is written in kOzSlices balanced base-256 digits,
//    Q = sum_{s=0..5} A_s 256^(5-s), A_0 in [-256, 256], A_s in [-128, 127]
//    for s > 0: small integers that FP16 holds exactly;
//  * Delta X = 2^(e_i + f_c - 16) sum_l 2^(-8 l) L_l with the level sums
//    L_l = sum_{s+t=l} A_s B_t over the levels l = 0..kOzSlices-1 (the
//    products of lower weight are dropped: each is below 2^-47 of the
//    fixed-point scale).  Every product of two digits is an integer below
//    2^16 in magnitude and every level sum over kOzPeriod consecutive K
//    elements stays below 2^24, so the tensor cores' FP32 accumulation adds
//    integers exactly; the accumulators are drained every kOzPeriod K
//    elements and combined in double-float arithmetic.
//
// The rounding to Q and the digit extraction use integer operations only
// (GB300 runs FP64 arithmetic at 1/64 of the FP32 rate).
#pragma once

#include <stdint.h>

namespace iptgb {

constexpr int kOzSlices = 6;      // digits per operand (48 bits)
constexpr int kOzPeriod = 128;    // K elements between accumulator drains
constexpr int kOzMaxCols = 64;    // columns per product launch
// Row / column exponent of a row that holds Inf or NaN: the product of that
// row (column) is NaN.
constexpr int kOzNonFinite = 0x7fffffff;

#if defined(__CUDACC__)
#define OZ_HD __host__ __device__ __forceinline__
#else
#define OZ_HD inline
#endif

// Smallest e with |v| < 2^e for the absolute-value bit pattern `absbits` of
// the largest |v| (0 for an all-zero row, kOzNonFinite for Inf / NaN).
OZ_HD int oz_exponent(uint64_t absbits)
{
    if (absbits == 0) return 0;
    const int E = (int)(absbits >> 52);
    if (E == 2047) return kOzNonFinite;
    if (E == 0) {
        // subnormal: absbits * 2^-1074 < 2^(p + 1 - 1074), p the top set bit
        int p = 0;
        while ((absbits >> (p + 1)) != 0) ++p;
        return p + 1 - 1074;
    }
    return E - 1022;  // 1.f * 2^(E - 1023) < 2^(E - 1022)
}

// The 48-bit fixed-point value round(v 2^(48 - e)) (round half away from
// zero) of a finite v with |v| < 2^e; 0 for non-finite v.
OZ_HD int64_t oz_fixed(double v, int e)
{
    uint64_t b;
#if defined(__CUDA_ARCH__)
    b = (uint64_t)__double_as_longlong(v);
#else
    __builtin_memcpy(&b, &v, sizeof(b));
#endif
    const bool neg = (b >> 63) != 0;
    b &= 0x7FFFFFFFFFFFFFFFULL;
    const int E = (int)(b >> 52);
    if (E == 2047 || b == 0 || e == kOzNonFinite) return 0;
    uint64_t M;
    int x;  // |v| = M * 2^x
    if (E == 0) {
        M = b;
        x = -1074;
    } else {
        M = (b & 0x000FFFFFFFFFFFFFULL) | 0x0010000000000000ULL;
        x = E - 1075;
    }
    const int sh = e - 48 - x;  // Q = M * 2^-sh
    uint64_t q;
    if (sh >= 60) {
        q = 0;
    } else if (sh > 0) {
        q = (M >> sh) + ((M >> (sh - 1)) & 1ULL);
    } else {
        q = M << (-sh);  // only for a row whose largest entry is subnormal
    }
    return neg ? -(int64_t)q : (int64_t)q;
}

// Balanced base-256 digits of a fixed-point value: q = sum_s d[s] 256^(5-s).
OZ_HD void oz_digits_of(int64_t q, int (&d)[kOzSlices])
{
#pragma unroll
    for (int s = kOzSlices - 1; s >= 1; --s) {
        const int64_t r = ((q + 128) & 255) - 128;
        d[s] = (int)r;
        q = (q - r) >> 8;  // exact: q - r is a multiple of 256
    }
    d[0] = (int)q;
}

// The same digits as oz_digits_of(oz_fixed(v, e)) in 32-bit integer
// arithmetic except one 64-bit shift: with q = H 2^24 + L (0 <= L < 2^24) the
// three low digits depend only on L (carry c in {0, 1} out of them) and the
// three high ones on H + c.
OZ_HD void oz_digits_fast(double v, int e, int (&d)[kOzSlices])
{
    uint64_t b;
#if defined(__CUDA_ARCH__)
    b = (uint64_t)__double_as_longlong(v);
#else
    __builtin_memcpy(&b, &v, sizeof(b));
#endif
    const uint32_t hi = (uint32_t)(b >> 32);
    const int E = (int)((hi >> 20) & 0x7FF);
    const int sh = E == 0 ? e - 48 + 1074 : e - 48 - (E - 1075);
    if (E == 2047 || e == kOzNonFinite || sh <= 0 || (b << 1) == 0) {
        oz_digits_of(oz_fixed(v, e), d);  // zero, non-finite, or a subnormal-scale row
        return;
    }
    uint32_t L;
    int32_t H;
    if (sh >= 60) {
        L = 0;
        H = 0;
    } else {
        const uint64_t M = E == 0 ? (b & 0x000FFFFFFFFFFFFFULL)
                                  : ((b & 0x000FFFFFFFFFFFFFULL) | 0x0010000000000000ULL);
        const uint64_t q = (M + (1ULL << (sh - 1))) >> sh;  // < 2^48 + 1
        const bool neg = (hi >> 31) != 0;
        const uint64_t qs = neg ? (uint64_t)0 - q : q;
        L = (uint32_t)qs & 0xFFFFFFu;
        H = (int32_t)((int64_t)qs >> 24);
    }
    int32_t t = (int32_t)L;
#pragma unroll
    for (int s = kOzSlices - 1; s >= 3; --s) {
        const int32_t r = ((t + 128) & 255) - 128;
        d[s] = r;
        t = (t - r) >> 8;
    }
    int32_t u = H + t;
#pragma unroll
    for (int s = 2; s >= 1; --s) {
        const int32_t r = ((u + 128) & 255) - 128;
        d[s] = r;
        u = (u - r) >> 8;
    }
    d[0] = u;
}

}  // namespace iptgb

#if defined(__CUDACC__)
#include <cuda_fp16.h>

namespace iptgb {

// FP16 values of two digits (|d| <= 256): 1536 + d has FP16 bit pattern
// 0x6600 + d (unit spacing in [1024, 2048)), and subtracting 1536 is exact.
__device__ __forceinline__ __half2 oz_digit_pair(int d0, int d1)
{
    const uint32_t bits = (uint32_t)(0x6600 + d0) | ((uint32_t)(0x6600 + d1) << 16);
    return __hsub2(*reinterpret_cast<const __half2 *>(&bits), __float2half2_rn(1536.0f));
}

// Write the kOzSlices digit slices of two neighbouring entries (v0, v1) of a
// row with exponent e: slice s goes to dst[s * slice_stride] (a __half2).
__device__ __forceinline__ void oz_store_pair(double v0, double v1, int e, __half2 *dst,
                                              size_t slice_stride)
{
    int a[kOzSlices], b[kOzSlices];
    oz_digits_fast(v0, e, a);
    oz_digits_fast(v1, e, b);
#pragma unroll
    for (int s = 0; s < kOzSlices; ++s) {
        dst[(size_t)s * slice_stride] = oz_digit_pair(a[s], b[s]);
    }
}

}  // namespace iptgb
#endif
