// Host check of the certified fixed-point helpers (kernels_gb300/csrc/prk_fixed.cuh) against the
// host's binary64 arithmetic: from_fixed / to_fixed round trips, classify on ordinary and special
// values, and certify's bounds. Prints "bad=<count>" and exits non-zero on any mismatch.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "prk_fixed.cuh"

using namespace prk::fx;

static uint64_t bits(double d)
{
    uint64_t b;
    std::memcpy(&b, &d, 8);
    return b;
}

static double dbl(uint64_t b)
{
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

int main()
{
    std::mt19937_64 g(20260101);
    int bad = 0;
    for (int t = 0; t < 1000000; ++t) {
        int64_t x = static_cast<int64_t>(g() >> (11 + g() % 52));
        if (g() & 1) x = -x;
        const int unit = static_cast<int>(g() % 80) - 60;
        const double want = std::ldexp(static_cast<double>(x), unit);
        if (dbl(from_fixed(x, unit)) != want || (x == 0 && from_fixed(x, unit) != 0)) bad++;
        int lo, hi;
        classify(bits(want), lo, hi);
        if (x != 0) {
            if (to_fixed(bits(want), unit) != x) bad++;
            if (lo < unit || hi != std::ilogb(want)) bad++;
        }
    }
    int lo, hi;
    classify(bits(-0.0), lo, hi);
    bad += lo != NOT_FIXED;
    classify(bits(5e-324), lo, hi);
    bad += lo != NOT_FIXED;
    classify(bits(INFINITY), lo, hi);
    bad += lo != NOT_FIXED;
    classify(bits(NAN), lo, hi);
    bad += lo != NOT_FIXED;
    classify(bits(0.0), lo, hi);
    bad += lo != ZERO_LO || hi != ZERO_HI;
    classify(bits(6.0), lo, hi);
    bad += lo != 1 || hi != 2;
    classify(bits(-0.375), lo, hi);
    bad += lo != -3 || hi != -2;
    // certify: integers below 2^15 with the star R=2 coefficients (shift 3, sum |c| = 12) pass;
    // a span that would overflow 2^53 units fails; a special value fails
    bad += certify(0, 14, 3, 12, 1) != 0;
    bad += certify(-4, 14, 3, 12, 8) != -4;
    bad += certify(0, 50, 3, 12, 1) != NOT_FIXED;
    bad += certify(NOT_FIXED, 3, 3, 12, 1) != NOT_FIXED;
    bad += certify(ZERO_LO, ZERO_HI, 3, 12, 1) != 0;
    std::printf("bad=%d\n", bad);
    return bad != 0;
}
