// Exactness-certified fixed-point evaluation of the binary64 stencil.
//
// GB300 issues binary64 arithmetic at about 1/73 of its FP32/INT32 rate, so the FP64 form avoids
// the DP pipe wherever it can prove the result would be the same bits. For stencils whose weights
// are all +-2^-k (star R=1,2 and grid R=1) every product w*v is exact in binary64. If, in addition,
// every value of an input tile is an integer multiple of 2^L and the tile's magnitudes are bounded
// so that sum |w*v| < 2^(53+L-s) (s = the largest weight shift), then every partial sum of the
// reference's left-to-right evaluation is an integer multiple of 2^(L-s) below 2^53 units: each
// rounding step is exact and the reference result equals the exact sum. That sum is computed in
// integer arithmetic and converted to binary64 once. A tile that fails the check is evaluated with
// binary64 instructions in the reference order, so both routes give identical bits for every input.
//
// The helpers here are plain integer bit manipulation on the IEEE-754 encoding; they compile for
// host and device so the host tests can check them against the host's binary64 arithmetic.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define PRK_HD __host__ __device__ __forceinline__
#else
#define PRK_HD inline
#endif

namespace prk {
namespace fx {

constexpr uint64_t SIGN = 0x8000000000000000ull;
constexpr uint64_t MANT = 0x000FFFFFFFFFFFFFull;
constexpr uint64_t HIDDEN = 0x0010000000000000ull;
constexpr int NOT_FIXED = 1 << 20;  // marker exponent for values that cannot be certified
constexpr int ZERO_LO = 1 << 19;    // lowest-bit exponent reported for +0 (neutral for a min)
constexpr int ZERO_HI = -(1 << 19); // highest-bit exponent reported for +0 (neutral for a max)

PRK_HD int clz64(uint64_t x)
{
#ifdef __CUDA_ARCH__
    return __clzll(static_cast<long long>(x));
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

PRK_HD int ctz64(uint64_t x)
{
#ifdef __CUDA_ARCH__
    return __ffsll(static_cast<long long>(x)) - 1;
#else
    return x ? __builtin_ctzll(x) : -1;
#endif
}

// Exponents of the lowest and highest set bit of a binary64 value: v = +-m * 2^e with m odd, then
// lo = e and hi = floor(log2|v|). +0 gives (ZERO_LO, ZERO_HI). -0, subnormals, infinities and
// NaNs give lo = NOT_FIXED: they are never certified (their exact-arithmetic image would lose the
// sign of zero or leave the normal range).
PRK_HD void classify(uint64_t b, int& lo, int& hi)
{
    if ((b << 1) == 0) {
        if (b & SIGN) {
            lo = NOT_FIXED;
            hi = NOT_FIXED;
        } else {
            lo = ZERO_LO;
            hi = ZERO_HI;
        }
        return;
    }
    const int bexp = static_cast<int>((b >> 52) & 0x7FF);
    if (bexp == 0 || bexp == 0x7FF) {
        lo = NOT_FIXED;
        hi = NOT_FIXED;
        return;
    }
    const uint64_t m = (b & MANT) | HIDDEN;
    hi = bexp - 1023;
    lo = hi - 52 + ctz64(m);
}

// The integer V with v = V * 2^unit, for a value already certified (lo >= unit, |V| < 2^63).
PRK_HD int64_t to_fixed(uint64_t b, int unit)
{
    if ((b << 1) == 0) return 0;
    const int bexp = static_cast<int>((b >> 52) & 0x7FF);
    const uint64_t m = (b & MANT) | HIDDEN;
    const int sh = bexp - 1075 - unit;  // v = m * 2^(bexp-1075)
    const uint64_t a = sh >= 0 ? (m << sh) : (m >> (-sh));
    return (b & SIGN) ? -static_cast<int64_t>(a) : static_cast<int64_t>(a);
}

// binary64 encoding of x * 2^unit, exact for |x| < 2^53 and a result in the normal range.
PRK_HD uint64_t from_fixed(int64_t x, int unit)
{
    if (x == 0) return 0;
    const uint64_t s = x < 0 ? SIGN : 0;
    const uint64_t a = x < 0 ? static_cast<uint64_t>(-x) : static_cast<uint64_t>(x);
    const int msb = 63 - clz64(a);
    const uint64_t m = a << (52 - msb);  // hidden bit at position 52
    // (bexp-1) << 52 plus m (whose hidden bit carries into the exponent field) = bexp << 52 | frac
    return s | ((static_cast<uint64_t>(msb + unit + 1022) << 52) + m);
}

// The encoding of a + 1 for a positive whole number 1 <= a < 2^53 (encoding b): a's encoding plus
// one unit of the integer position, the mantissa's 2^(1075 - e) bit, whose carry steps the
// exponent when the mantissa overflows (a = 2^k - 1). Returns false, leaving *r alone, for any other
// value (negative, fractional, zero, subnormal, at or above 2^53, infinite or NaN).
PRK_HD bool inc_whole(uint64_t b, uint64_t* r)
{
    const int e = static_cast<int>(b >> 52);  // >= 2048 for negative values
    if (e < 1023 || e > 1075) return false;
    const uint64_t unit = 1ull << (1075 - e);
    if (b & (unit - 1)) return false;
    *r = b + unit;
    return true;
}

PRK_HD int clz32(uint32_t x)
{
#ifdef __CUDA_ARCH__
    return __clz(static_cast<int>(x));
#else
    return x ? __builtin_clz(x) : 32;
#endif
}

// mul_whole20 (below) with the weight pre-split, as a table entry holds it: w1 = the low 32 bits of
// w's significand W, w2 = its high 21 bits with the hidden bit, hib = w's sign and biased exponent
// field as in the encoding's high word.
PRK_HD uint64_t mul_whole20_split(uint32_t w1, uint32_t w2, uint32_t hib, int32_t v)
{
    const uint32_t vs = static_cast<uint32_t>(v) & 0x80000000u;
    const uint32_t a = static_cast<uint32_t>(v < 0 ? -v : v);
    const uint64_t x = static_cast<uint64_t>(w1) * a;
    const uint64_t y = static_cast<uint64_t>(w2) * a;
    const uint64_t mid = (x >> 32) + (y & 0xFFFFFFFFull);
    const uint32_t p0 = static_cast<uint32_t>(x), p1 = static_cast<uint32_t>(mid);
    const uint32_t p2 = static_cast<uint32_t>((y >> 32) + (mid >> 32));
    const int sh = (p2 ? 96 - clz32(p2) : 64 - clz32(p1)) - 53;
    const uint32_t q_lo = static_cast<uint32_t>(((static_cast<uint64_t>(p1) << 32) | p0) >> (sh & 63));
    const uint32_t q_hi = static_cast<uint32_t>(((static_cast<uint64_t>(p2) << 32) | p1) >> (sh & 63));
    const uint32_t mask = (1u << (sh & 31)) - 1u, rem = p0 & mask;
    // round to nearest-even: add half - 1 + (lowest kept bit) to the bits below, carry into q
    const uint32_t bump = (rem + (mask >> 1) + (sh > 0 ? (q_lo & 1u) : 0u)) >> (sh & 31);
    const uint64_t q = ((static_cast<uint64_t>(q_hi) << 32) | q_lo) + (sh > 0 ? bump : 0u);
    const uint32_t ovf = static_cast<uint32_t>(q >> 53);  // 1 when rounding carried to 2^53
    const uint32_t hi = ((hib ^ vs) & 0x80000000u) | ((hib & 0x7FF00000u) + ((static_cast<uint32_t>(sh) + ovf) << 20)) |
                        (static_cast<uint32_t>(q >> (32 + ovf)) & 0xFFFFFu);
    const uint32_t lo = static_cast<uint32_t>(q >> ovf);
    return v == 0 ? static_cast<uint64_t>(hib & 0x80000000u) << 32 : (static_cast<uint64_t>(hi) << 32) | lo;
}

// Bits of fl(w * v), the binary64 product rounded to nearest-even, for a normal binary64 w (encoding
// wb, biased exponent at most 2025) and a whole number |v| < 2^20, from integer operations on w's
// 53-bit significand W: W * |v| < 2^73 is formed as three 32-bit words from two 32 x 32 -> 64-bit
// products, its top 53 bits are taken with two 64-bit funnel shifts and rounded on the bits below
// (the half-way case to the even neighbour). v = 0 gives the zero of w's sign (w * +0).
PRK_HD uint64_t mul_whole20(uint64_t wb, int32_t v)
{
    const uint32_t whi = static_cast<uint32_t>(wb >> 32);
    return mul_whole20_split(static_cast<uint32_t>(wb), (whi & 0xFFFFFu) | 0x100000u, whi & 0xFFF00000u, v);
}

// Certification of a tile whose values have lowest-bit exponents >= lo_min and highest-bit
// exponents <= hi_max, for a stencil with weight shift `shift` and coefficient L1 norm `coef_l1`
// (sum |w| * 2^shift), and `steps` in += 1 updates applied to the tile before its last use.
// Returns the unit exponent L (values are integers in units of 2^L) or NOT_FIXED.
//   - L = min(lo_min, 0): 1.0 must be a whole number of units for the in += 1 update;
//   - L >= -51 and L - shift >= -960: units stay far inside the normal range;
//   - (max|V| + steps * 2^-L) * coef_l1 < 2^53: every partial sum of every application, and every
//     updated value, is an integer below 2^53 units (bounded via 2^(hi_max+1) > max|v|).
PRK_HD int certify(int lo_min, int hi_max, int shift, int64_t coef_l1, int steps)
{
    if (lo_min >= NOT_FIXED || hi_max >= NOT_FIXED || steps < 0 || steps > 1024 || coef_l1 < 1) return NOT_FIXED;
    const int L = lo_min < 0 ? lo_min : 0;
    if (L < -51 || L - shift < -960 || hi_max > 60) return NOT_FIXED;
    const int span = hi_max == ZERO_HI ? 0 : hi_max + 1 - L;  // max|V| < 2^span
    if (span > 52) return NOT_FIXED;
    // integer-only bound: vmax < floor(2^53 / coef_l1) implies vmax * coef_l1 < 2^53
    const uint64_t vmax = (1ull << span) + static_cast<uint64_t>(steps) * (1ull << (-L));
    if (vmax >= (1ull << 53) / static_cast<uint64_t>(coef_l1)) return NOT_FIXED;
    return L;
}

}  // namespace fx
}  // namespace prk
