// Host check of the certified fixed-point helpers (kernels_gb300/csrc/prk_fixed.cuh) against the
// host's binary64 arithmetic: from_fixed / to_fixed round trips, classify on ordinary and special
// values, and certify's bounds. Prints "bad=<count>" and exits non-zero on any mismatch.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

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
    // mul_whole20 against the host's binary64 multiply: the stencil weights and random normal w,
    // random and edge whole numbers v with |v| < 2^20
    {
        std::vector<double> ws;
        for (int R = 1; R <= 5; ++R)
            for (int j = 1; j <= R; ++j) {
                ws.push_back(1.0 / (2.0 * j * R));
                ws.push_back(-1.0 / (2.0 * j * R));
                ws.push_back(1.0 / (4.0 * j * (2.0 * j - 1) * R));
                ws.push_back(-1.0 / (4.0 * j * R));
            }
        for (int t = 0; t < 2000; ++t) {
            double w = std::ldexp(1.0 + static_cast<double>(g() >> 12) * 0x1p-52, static_cast<int>(g() % 200) - 100);
            ws.push_back(g() & 1 ? -w : w);
        }
        std::vector<int32_t> vs = {0, 1, -1, 2, 3, 7, 2147483647, -2147483647};
        for (int k = 1; k < 31; ++k) {
            vs.push_back((1 << k) - 1);
            vs.push_back(1 << k);
            vs.push_back(-(1 << k) + 1);
            vs.push_back((1 << k) + 1);
        }
        for (int t = 0; t < 3000; ++t) {
            const int32_t v = static_cast<int32_t>(g() >> (33 + g() % 31));
            vs.push_back(g() & 1 ? -v : v);
        }
        long checked = 0;
        for (double w : ws)
            for (int32_t v : vs) {
                const double want = w * static_cast<double>(v);
                if (v <= -(1 << 20) || v >= (1 << 20)) continue;
                bad += mul_whole20(bits(w), v) != bits(want);
                {
                    const uint64_t wb = bits(w);
                    const uint32_t w1 = static_cast<uint32_t>(wb), w2 = static_cast<uint32_t>((wb >> 32) & 0xFFFFFu) | 0x100000u;
                    bad += mul_whole20_split(w1, w2, static_cast<uint32_t>(wb >> 32) & 0xFFF00000u, v) != bits(want);
                }
                ++checked;
            }
        // every |v| < 2^20 against a few weights
        for (double w : {1.0 / 6.0, -1.0 / 18.0, 1.0 / 48.0, -1.0 / 100.0, 1.0 / 30.0})
            for (int32_t v = -(1 << 20) + 1; v < (1 << 20); ++v) {
                bad += mul_whole20(bits(w), v) != bits(w * static_cast<double>(v));
                const uint64_t wb = bits(w);
                const uint32_t w1 = static_cast<uint32_t>(wb), w2 = static_cast<uint32_t>((wb >> 32) & 0xFFFFFu) | 0x100000u;
                bad += mul_whole20_split(w1, w2, static_cast<uint32_t>(wb >> 32) & 0xFFF00000u, v) != bits(w * static_cast<double>(v));
                ++checked;
            }
        std::printf("mul_whole20 checked=%ld\n", checked);
    }
    // inc_whole against the host's a + 1.0: random whole numbers below 2^53, 2^k - 1 (the carry into
    // the exponent), powers of two, and values it must refuse (then a + 1.0 is left to binary64)
    {
        std::vector<double> as = {0.0, -0.0, -1.0, -5.0, 0.5, 1.5, 0x1p53, 0x1p52 + 2.0, INFINITY, NAN, 5e-324, 1.0};
        for (int k = 1; k < 54; ++k) {
            as.push_back(std::ldexp(1.0, k) - 1.0);
            as.push_back(std::ldexp(1.0, k));
        }
        for (int t = 0; t < 200000; ++t) as.push_back(static_cast<double>(g() >> 11));
        for (int t = 0; t < 1000; ++t) as.push_back(std::ldexp(static_cast<double>(g() >> 11), -20) * (g() & 1 ? 1 : -1));
        long checked = 0, certified = 0;
        for (double a : as) {
            uint64_t r;
            if (inc_whole(bits(a), &r)) {
                bad += r != bits(a + 1.0);
                ++certified;
            } else {
                bad += (a >= 1.0 && a < 0x1p53 && a == std::floor(a));  // a whole number it should take
            }
            ++checked;
        }
        std::printf("inc_whole checked=%ld certified=%ld\n", checked, certified);
    }
    // The 96-bit fixed-point chain against the host's binary64 chain: fx96_from_bits of each term,
    // fx96_acc_round for every add (or subtract), fx96_to_bits at the end, against
    // ((p1 + p2) + ...) in binary64. Terms: products fl(w * v) of every PRK weight with whole numbers
    // |v| < 2^20 (the stencil chains), and random multiples of 2^-62 below 2^20 with few significant
    // bits, whose sums fall on rounding ties often. The domain is |sum| < 2^21 (the strict stencils'
    // weights sum to at most 1.25 in magnitude and their values stay below 2^20); a chain is checked
    // until it leaves it.
    {
        std::vector<double> ws;
        for (int R = 1; R <= 5; ++R)
            for (int m = 1; m <= R; ++m) {
                ws.push_back(1.0 / (2.0 * m * R));
                ws.push_back(1.0 / (4.0 * m * (2.0 * m - 1) * R));
                ws.push_back(1.0 / (4.0 * m * R));
            }
        long checked = 0;
        auto run_chain = [&](const std::vector<double>& terms, const std::vector<int>& neg) {
            double want = neg[0] ? -terms[0] : terms[0];
            uint32_t x0, x1, x2;
            fx96_from_bits(bits(want), x0, x1, x2);
            bool allneg0 = bits(want) == SIGN;
            for (size_t k = 1; k < terms.size(); ++k) {
                uint32_t p0, p1, p2;
                fx96_from_bits(bits(terms[k]), p0, p1, p2);
                if (neg[k]) {
                    fx96_acc_round<true>(x0, x1, x2, p0, p1, p2);
                    want = want - terms[k];
                    allneg0 = allneg0 && bits(-terms[k]) == SIGN;
                } else {
                    fx96_acc_round<false>(x0, x1, x2, p0, p1, p2);
                    want = want + terms[k];
                    allneg0 = allneg0 && bits(terms[k]) == SIGN;
                }
                if (std::fabs(want) >= 0x1p21) break;  // outside the domain (the stencils stay below 2^21)
                bad += fx96_to_bits(x0, x1, x2, allneg0) != bits(want);
                ++checked;
            }
        };
        for (int t = 0; t < 300000; ++t) {
            const int len = 1 + static_cast<int>(g() % 110);
            const int32_t vbase = static_cast<int32_t>(g() % (t % 3 == 0 ? 64 : (1u << 20)));
            std::vector<double> terms;
            std::vector<int> neg;
            for (int k = 0; k < len; ++k) {
                int32_t v = vbase + static_cast<int32_t>(g() % 200) - 100;
                if (v <= -(1 << 20) || v >= (1 << 20)) v = 0;
                const double w = ws[g() % ws.size()];
                terms.push_back(w * static_cast<double>(v < 0 ? -v : v));
                neg.push_back((v < 0) ^ static_cast<int>(g() & 1));
            }
            run_chain(terms, neg);
        }
        for (int t = 0; t < 300000; ++t) {
            const int len = 2 + static_cast<int>(g() % 40);
            std::vector<double> terms;
            std::vector<int> neg;
            for (int k = 0; k < len; ++k) {
                const int sig = 1 + static_cast<int>(g() % 53);
                const uint64_t mant = (g() >> (64 - sig)) | (1ull << (sig - 1));
                const int e = static_cast<int>(g() % 30) - 10;  // leading bit 2^-10 .. 2^19
                double v = std::ldexp(static_cast<double>(mant), e - (sig - 1));
                if (g() % 17 == 0) v = 0.0;
                terms.push_back(v);
                neg.push_back(static_cast<int>(g() & 1));
            }
            run_chain(terms, neg);
        }
        // a chain of -0 terms, and cancellation to +0
        run_chain({0.0, 0.0, 0.0}, {1, 1, 1});
        run_chain({0.0, 0.0}, {1, 0});
        run_chain({1.0 / 6.0 * 5, 1.0 / 6.0 * 5}, {0, 1});
        std::printf("fx96 chain steps checked=%ld\n", checked);
    }
    std::printf("bad=%d\n", bad);
    return bad != 0;
}
