// fpconv.cuh - double -> float conversions on the integer pipe.
//
// On GB300 the FP64 pipe (about 2 operations per clock per SM) also executes
// the F2F conversions between double and float, so a pass that converts every
// entry of a large FP64 matrix is bound by that pipe, not by HBM.  These
// helpers produce the same bits with 32-bit integer operations for the
// entries that occur in practice (|h| a normal float and h - float(h) a
// normal float too); the others take the FP64 instructions.
//
//   split_double(h) -> (hi, lo):  hi = RN_float(h), lo = RN_float(h - hi),
//   bit-identical to __double2float_rn(h) and __double2float_rn(h - (double)hi)
//   (h - hi is exact in double, so lo is the rounding of the exact remainder).
#pragma once

#include <stdint.h>

namespace iptgb {

#if defined(__CUDACC__)
#define IPTGB_HD __host__ __device__ __forceinline__
#else
#define IPTGB_HD inline
#endif

IPTGB_HD int clz32_hd(uint32_t x)
{
#if defined(__CUDA_ARCH__)
    return __clz((int)x);
#else
    return x == 0 ? 32 : __builtin_clz(x);
#endif
}

// Bits of (hi, lo) for the common case; returns false when the entry needs
// the FP64 instructions (|h| outside the normal float range, an overflow of
// hi, or a remainder below the normal float range).
IPTGB_HD bool split_double_bits(uint64_t b, uint32_t *hi_bits, uint32_t *lo_bits)
{
    const uint32_t h32 = (uint32_t)(b >> 32);
    const uint32_t l32 = (uint32_t)b;
    const uint32_t e = (h32 >> 20) & 0x7FFu;  // biased double exponent
    // |h| in [2^-126, 2^128): e - 1023 in [-126, 127]
    if (e - 897u >= 254u) return false;
    const uint32_t sign = h32 & 0x80000000u;
    // truncated float: exponent e - 896, top 23 of the 52 mantissa bits
    const uint32_t f = sign | ((e - 896u) << 23) | ((h32 & 0xFFFFFu) << 3) | (l32 >> 29);
    const uint32_t rem = l32 & 0x1FFFFFFFu;  // the 29 dropped bits
    const uint32_t inc = (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
    const uint32_t hb = f + inc;  // a carry moves into the exponent, as rounding does
    if ((hb & 0x7F800000u) == 0x7F800000u) return false;  // rounded to infinity
    *hi_bits = hb;
    // h - hi = sign * d * 2^(E - 52), d = rem - inc * 2^29, |d| <= 2^28
    const int32_t d = (int32_t)rem - (int32_t)(inc << 29);
    if (d == 0) {
        *lo_bits = 0u;  // x - x = +0 under round-to-nearest
        return true;
    }
    const uint32_t ad = (uint32_t)(d < 0 ? -d : d);
    const uint32_t lsign = sign ^ (d < 0 ? 0x80000000u : 0u);
    const int t = 31 - clz32_hd(ad);               // 0..28
    const int biased = t + (int)e - 948;           // float exponent of the remainder
    if (biased < 1) return false;                  // float subnormal remainder
    uint32_t lb;
    if (t <= 23) {
        lb = lsign | ((uint32_t)biased << 23) | ((ad << (23 - t)) & 0x7FFFFFu);
    } else {
        const int s = t - 23;  // 1..5 dropped bits
        const uint32_t mant = ad >> s;
        const uint32_t r = ad & ((1u << s) - 1u);
        const uint32_t half = 1u << (s - 1);
        lb = lsign | ((uint32_t)biased << 23) | (mant & 0x7FFFFFu);
        lb += (r > half || (r == half && (mant & 1u))) ? 1u : 0u;
    }
    *lo_bits = lb;
    return true;
}

#undef IPTGB_HD

}  // namespace iptgb
