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
// the 106-bit significand product is formed from the 64x64-bit product of
// ma << 11 and mb << 11 (high word exact, low word only as a sticky bit),
// normalised by one position when it is >= 2^105, and rounded to 53 bits
// with round-to-nearest-even on (round bits, sticky).  Operands that are
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

HSMU_HD uint64_t mulhi64(uint64_t x, uint64_t y) {
#ifdef __CUDA_ARCH__
    return __umul64hi(x, y);
#else
    return (uint64_t)(((unsigned __int128)x * y) >> 64);
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

// a * b rounded to nearest even, bit-identical to the IEEE multiply.
HSMU_HD double dmul_int(double a, double b) {
    const uint64_t ua = dbits(a), ub = dbits(b);
    const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu;
    const uint32_t eb = (uint32_t)(ub >> 52) & 0x7ffu;
    // biased exponent if the significand product is in [1, 2)
    const int e0 = (int)ea + (int)eb - 1023;
    if (ea - 1u >= 2046u || eb - 1u >= 2046u || (unsigned)(e0 - 1) >= 2045u) return native_dmul(a, b);
    const uint64_t frac = (1ull << 52) - 1ull;
    const uint64_t x = ((ua & frac) | (1ull << 52)) << 11;  // ma * 2^11, top bit set
    const uint64_t y = ((ub & frac) | (1ull << 52)) << 11;
    const uint64_t hi = mulhi64(x, y);   // floor(ma*mb / 2^42), in [2^62, 2^64)
    const uint64_t lo = x * y;           // remaining bits (sticky only)
    const uint32_t top = (uint32_t)(hi >> 63);  // 1 when ma*mb >= 2^105
    const uint32_t sh = 10u + top;              // bits below the 53-bit significand
    uint64_t m = hi >> sh;
    const uint64_t rem = hi & ((1ull << sh) - 1ull);
    const uint64_t half = 1ull << (sh - 1u);
    const uint64_t up = (rem > half) | ((rem == half) & ((lo != 0ull) | (m & 1ull)));
    m += up;
    int e = e0 + (int)top;
    // m == 2^53 after rounding up an all-ones significand: renormalise
    const uint64_t carry = m >> 53;
    m >>= carry;
    e += (int)carry;
    if (e >= 2047) return native_dmul(a, b);  // overflow to infinity
    return bitsd(((ua ^ ub) & (1ull << 63)) | ((uint64_t)e << 52) | (m & frac));
}

}  // namespace hsmu
