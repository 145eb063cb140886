// Exact binary64 addition on the 32-bit integer pipe.
//
// GB300's FP64 pipe retires about 1.8 lane operations per clock per SM, the
// integer pipe 64: an FP64 stencil sweep keeps the FP64 pipe busy while the
// integer pipe idles.  dadd_same_sign_bits computes a + b, rounded to
// nearest even exactly as the FP64 adder does (the same bits), from the
// operands' bit patterns with integer instructions only.  It covers the case
// that dominates the neighbour sums of a smooth field -- both operands of
// one sign, exponents at most 10 apart, the smaller exponent field in
// [1, 2035] (magnitudes from 2^-1022 to about 2^1013) -- and reports every
// other case (zeros, subnormals, infinities, NaNs, opposite signs, distant
// exponents, huge magnitudes) through `ok`, for the caller to add in FP64
// instead.
//
// Method (textbook IEEE addition with guard bits): order the operands by
// magnitude, place the larger significand (hidden bit included) at bits
// 62..10 of a 64-bit word and the smaller one at bits 62-d..10-d, d <= 10
// the exponent difference, so that no bit is shifted out and the sum is
// exact; add; round to nearest even at bit 10, or at bit 11 when the sum
// carried into bit 63; pack: the rounded significand's hidden bit is added
// into the exponent field, so a rounding carry raises the exponent by
// itself.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define SCAFES_HD __host__ __device__ __forceinline__
#else
#define SCAFES_HD inline
#endif

namespace scafes {

SCAFES_HD uint64_t dadd_same_sign_bits(uint64_t a, uint64_t b, bool& ok) {
    const uint32_t ah = (uint32_t)(a >> 32), al = (uint32_t)a;
    const uint32_t bh = (uint32_t)(b >> 32), bl = (uint32_t)b;
    // One sign: the larger high word has the larger (or the same) exponent.
    const bool a_big = ah >= bh;
    const uint32_t hh = a_big ? ah : bh, hl = a_big ? al : bl;
    const uint32_t lh = a_big ? bh : ah, ll = a_big ? bl : al;
    const uint32_t d = (hh >> 20) - (lh >> 20);  // the exponent difference when the signs agree
    // The smaller exponent in [1, 2035] and d <= 10.  With opposite signs d
    // is 2048 + ea - eb, which is above 10 for any eb <= 2035, so the range
    // test covers the sign test; the larger exponent is at most 2045.
    ok = d <= 10u && (lh & 0x7fffffffu) - 0x00100000u < 0x7f300000u;
    const uint32_t mah = (hh & 0x000fffffu) | 0x00100000u;
    const uint32_t mbh = (lh & 0x000fffffu) | 0x00100000u;
    uint32_t pb = 1u << ((10u - d) & 31u);
#if defined(__CUDA_ARCH__)
    // Keeps the alignment a multiply by 2^(10-d) (the FMA pipe) rather than
    // a shift (the integer ALU, which the adder keeps busier).
    asm("" : "+r"(pb));
#endif
    // ma * 2^10 + mb * 2^(10-d): exact, below 2^64.
    uint64_t s = (uint64_t)hl * 1024u + (uint64_t)ll * pb;
    s += (uint64_t)(mah * 1024u + mbh * pb) << 32;
    const uint32_t c = (uint32_t)(s >> 63);
    const uint32_t sh = 10u + c;
    // + (half - 1) + the last kept bit: rounds half to even.
    s += (uint64_t)((0x1ffu << c) + c + (((uint32_t)s >> sh) & 1u));
    const uint64_t m = s >> sh;  // 53 bits, or 2^53 after a rounding carry
    return ((uint64_t)((hh & 0xfff00000u) + (c << 20) - 0x00100000u) << 32) + m;
}

}  // namespace scafes
