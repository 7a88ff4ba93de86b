// Host check of the integer-pipe double multiply (hsmu_dmul.cuh) against the
// IEEE hardware multiply: random bit patterns (all exponents, specials),
// values in (-1, 1), and short significands that make exact products and
// round-half ties frequent.  Prints "ok <count>" or the first mismatch.
#include <cmath>
#include <cstdio>
#include <cstdint>

#include "hsmu_dmul.cuh"

static uint64_t s = 0x9E3779B97F4A7C15ull;
static uint64_t rnd() {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return s;
}

static bool same(double x, double y) {
    if (std::isnan(x) && std::isnan(y)) return true;
    return hsmu::dbits(x) == hsmu::dbits(y);
}

int main(int argc, char **argv) {
    long n = argc > 1 ? atol(argv[1]) : 2000000;
    long checked = 0;
    for (long i = 0; i < n; i++) {
        double a, b;
        switch (i % 6) {
        case 5: {  // products just below a power of two: rounding carries out of the significand
            uint64_t ma = (1ull << 52) + (rnd() >> 12);
            if (ma < 6369051672525773ull) ma += 6369051672525773ull - (1ull << 52);
            if (ma >= (1ull << 53)) ma = (1ull << 53) - 1;
            unsigned __int128 target = ((unsigned __int128)1 << 105) - 1;
            uint64_t mb = (uint64_t)(target / ma) - (rnd() % 3);
            if (mb >= (1ull << 53)) mb = (1ull << 53) - 1;
            a = ldexp((double)ma, -52);
            b = ldexp((double)mb, -52 + (int)(rnd() % 40) - 20);
            break;
        }
        case 0:
            a = hsmu::bitsd(rnd());
            b = hsmu::bitsd(rnd());
            break;
        case 1: {
            a = (double)(rnd() >> 11) * 0x1p-53 * 2.0 - 1.0;
            b = (double)(rnd() >> 11) * 0x1p-53 * 2.0 - 1.0;
            break;
        }
        case 2: {  // short significands: ties and exact products
            int bits = 24 + (int)(rnd() % 8);
            uint64_t ma = (rnd() >> (64 - bits)) | (1ull << (bits - 1));
            uint64_t mb = (rnd() >> (64 - bits)) | (1ull << (bits - 1));
            int ex = (int)(rnd() % 200) - 100, ey = (int)(rnd() % 200) - 100;
            a = ldexp((double)ma, ex) * ((rnd() & 1) ? -1.0 : 1.0);
            b = ldexp((double)mb, ey);
            break;
        }
        case 3: {  // exponent edges: results near overflow / underflow
            a = ldexp(1.0 + (double)(rnd() >> 12) * 0x1p-52, (int)(rnd() % 2100) - 1050);
            b = ldexp(1.0 + (double)(rnd() >> 12) * 0x1p-52, (int)(rnd() % 2100) - 1050);
            break;
        }
        default: {  // all-ones significands (rounding carries into the exponent)
            a = hsmu::bitsd((rnd() & 0x800FFFFF00000000ull) | 0x3FEFFFFFFFFFFFFFull);
            b = hsmu::bitsd(0x3FF0000000000000ull | (rnd() >> 12));
            break;
        }
        }
        double want = a * b;
        double got = hsmu::dmul_int(a, b);
        if (!same(want, got)) {
            printf("mismatch %a * %a: want %a got %a\n", a, b, want, got);
            return 1;
        }
        checked++;
    }
    printf("ok %ld\n", checked);
    return 0;
}
