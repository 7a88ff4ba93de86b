// Exact IEEE-754 binary64 multiplication (round to nearest, ties to even) on
// the integer pipe.
//
// Why: GB300 runs FP64 arithmetic at ~1.6 lane-ops/clk/SM (DADD, DMUL and
// DFMA alike) against ~100+ int32 lane-ops/clk/SM.  The numeric phase needs
// one multiply and one add per intermediate product, both on the FP64 pipe.
// Computing the multiply on the integer pipe with ~50 integer instructions
// leaves the FP64 pipe only the add, which roughly halves the FP64-pipe time
// per product.  The result is bit-identical to the hardware multiply.
//
// Method (textbook IEEE multiplication): with both operands normal,
//   a * b = (ma * mb) * 2^(ea + eb - 2*1023 - 104),  ma, mb in [2^52, 2^53),
// the exact 106-bit significand product is formed from 32-bit partial
// products, normalised by one position when it is >= 2^105, and rounded to
// 53 bits with round-to-nearest-even on (round bit, sticky bits).  Operands that are
// zero, subnormal, infinite or NaN, and products whose exponent leaves the
// normal range, take the hardware multiply instead, so every input gives the
// IEEE result.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define HSMU_HD __host__ __device__ __forceinline__
#else
#define HSMU_HD inline
#endif

namespace hsmu {

HSMU_HD uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, 8);
    return u;
#endif
}

HSMU_HD double bitsd(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, 8);
    return x;
#endif
}

HSMU_HD double native_dmul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    volatile double r = a * b;  // host: plain IEEE multiply (the file is built without FMA contraction)
    return r;
#endif
}

HSMU_HD uint64_t mulwide32(uint32_t x, uint32_t y) { return (uint64_t)x * (uint64_t)y; }

// a * b rounded to nearest even, bit-identical to the IEEE multiply.
// The 106-bit significand product is assembled from four 32 x 32 -> 64-bit
// partial products (one wide multiply-add each on the integer pipe) of the
// significands split as ma = ma_hi * 2^32 + ma_lo (ma_hi: 21 bits):
//   P = hh * 2^64 + (hl + lh) * 2^32 + ll = U * 2^64 + w1 * 2^32 + w0.
// P >> 52 (53 or 54 bits) is the significand before rounding; the bit below
// it rounds, the bits under that are the sticky bit.
HSMU_HD double dmul_int(double a, double b) {
    const uint64_t ua = dbits(a), ub = dbits(b);
    const uint32_t ah = (uint32_t)(ua >> 32), bh = (uint32_t)(ub >> 32);
    const uint32_t ea = (ah >> 20) & 0x7ffu;
    const uint32_t eb = (bh >> 20) & 0x7ffu;
    // biased exponent if the significand product is in [1, 2)
    const int e0 = (int)ea + (int)eb - 1023;
    if (ea - 1u >= 2046u || eb - 1u >= 2046u || (unsigned)(e0 - 1) >= 2045u) return native_dmul(a, b);
    const uint32_t xh = (ah & 0xfffffu) | 0x100000u, xl = (uint32_t)ua;
    const uint32_t yh = (bh & 0xfffffu) | 0x100000u, yl = (uint32_t)ub;
    const uint64_t ll = mulwide32(xl, yl);
    const uint64_t mid = mulwide32(xl, yh) + mulwide32(xh, yl);  // < 2^54
    const uint64_t hh = mulwide32(xh, yh);                        // < 2^42
    const uint64_t t = (ll >> 32) + (uint32_t)mid;                // < 2^33
    const uint32_t w0 = (uint32_t)ll, w1 = (uint32_t)t;
    const uint64_t U = hh + (mid >> 32) + (t >> 32);              // bits 64..105 of P, < 2^42
    const uint32_t top = (uint32_t)(U >> 41);                     // 1 when P >= 2^105
    uint64_t m = (U << 12) | (w1 >> 20);                          // P >> 52
    // round bit and sticky bits below the 53-bit significand
    const uint32_t rbit = top ? (uint32_t)(m & 1u) : (w1 >> 19) & 1u;
    const uint32_t sticky = (top ? (w1 & 0xfffffu) : (w1 & 0x7ffffu)) | w0;
    m >>= top;
    m += (uint64_t)(rbit & ((sticky != 0u) | (uint32_t)(m & 1u)));
    int e = e0 + (int)top;
    // m == 2^53 after rounding up an all-ones significand: renormalise
    const uint32_t carry = (uint32_t)(m >> 53);
    m >>= carry;
    e += (int)carry;
    if (e >= 2047) return native_dmul(a, b);  // overflow to infinity
    return bitsd(((ua ^ ub) & (1ull << 63)) | ((uint64_t)e << 52) | (m & ((1ull << 52) - 1ull)));
}

}  // namespace hsmu
