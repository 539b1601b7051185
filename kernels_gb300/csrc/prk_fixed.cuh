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
#include <cstring>

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

// ---- 96-bit fixed point for the strict-order sums ------------------------------------------------
// The stencils whose weights are not powers of two round every product and every partial sum of the
// reference's chain (((p1 + p2) + p3) + ...). On tiles of whole numbers |v| < 2^20 every product
// p = fl(w * v) of a PRK weight (|w| >= 1/900) is a multiple of 2^-62 (its lowest bit lies at most 52
// places below its leading bit, which is at or above 2^-10), and every partial sum, being the rounded
// sum of such multiples, is one too; all stay below 2^21 in magnitude (sum |w| <= 1.5, for grid
// R=2). Each value is then an integer of units 2^-62 below 2^83, held exactly in three 32-bit words
// as a two's-complement number, and a rounded binary64 add is: the exact integer sum, then rounding
// to 53 significant bits at the position its leading bit sets, to nearest with ties to the even
// neighbour. Both steps are integer instructions, so a chain can leave the binary64 pipe for the
// integer pipes and come back with the same bits (fx96_to_bits).
constexpr int FX96_F = 62;

// x = v * 2^62 for a binary64 v (encoding b) with |v| < 2^22 that is a multiple of 2^-62, or +-0.
PRK_HD void fx96_from_bits(uint64_t b, uint32_t& x0, uint32_t& x1, uint32_t& x2)
{
    x0 = x1 = x2 = 0;
    if ((b << 1) == 0) return;
    const int e = static_cast<int>((b >> 52) & 0x7FF);
    const uint64_t m = (b & MANT) | HIDDEN;  // v = m * 2^(e - 1075)
    const int sh = e - 1075 + FX96_F;       // v * 2^62 = m * 2^sh, sh <= 31 for |v| < 2^22
    uint64_t lo;
    uint32_t hi;
    if (sh >= 0) {
        lo = m << sh;
        hi = sh == 0 ? 0u : static_cast<uint32_t>(m >> (64 - sh));
    } else {
        lo = m >> (-sh);  // the bits shifted out are zero for a multiple of 2^-62
        hi = 0u;
    }
    if (b & SIGN) {  // two's-complement negation of the 96-bit value
        lo = ~lo + 1;
        hi = ~hi + (lo == 0 ? 1u : 0u);
    }
    x0 = static_cast<uint32_t>(lo);
    x1 = static_cast<uint32_t>(lo >> 32);
    x2 = hi;
}

// x = fl(x + p) (SUB: fl(x - p)) for 96-bit fixed-point values whose exact result lies below 2^83
// units (values below 2^21): the exact sum, then rounding to 53 significant bits, nearest-even. The
// position b of the rounding is the leading bit of |sum| less 52, at most 30, so only the low word
// is cut and the rounding increment carries into the others. Rounding the two's-complement value to a multiple of
// 2^b with ties to the even multiple gives the same result as rounding its magnitude and negating;
// the leading bit is read from the one's complement of a negative sum, which differs from the
// magnitude's only when the magnitude is a power of two (then nothing lies below b anyway).
template <bool SUB>
PRK_HD void fx96_acc_round(uint32_t& x0, uint32_t& x1, uint32_t& x2, uint32_t p0, uint32_t p1, uint32_t p2)
{
#ifdef __CUDA_ARCH__
    if (SUB)
        asm("sub.cc.u32 %0, %0, %3;\n\tsubc.cc.u32 %1, %1, %4;\n\tsubc.u32 %2, %2, %5;"
            : "+r"(x0), "+r"(x1), "+r"(x2)
            : "r"(p0), "r"(p1), "r"(p2));
    else
        asm("add.cc.u32 %0, %0, %3;\n\taddc.cc.u32 %1, %1, %4;\n\taddc.u32 %2, %2, %5;"
            : "+r"(x0), "+r"(x1), "+r"(x2)
            : "r"(p0), "r"(p1), "r"(p2));
#else
    const uint64_t a = (static_cast<uint64_t>(x1) << 32) | x0, pq = (static_cast<uint64_t>(p1) << 32) | p0;
    const uint64_t r = SUB ? a - pq : a + pq;
    const uint32_t c = SUB ? (a < pq ? 1u : 0u) : (r < a ? 1u : 0u);
    x2 = SUB ? x2 - p2 - c : x2 + p2 + c;
    x0 = static_cast<uint32_t>(r);
    x1 = static_cast<uint32_t>(r >> 32);
#endif
    // b = max(0, msb|sum| - 52). As |sum| < 2^83, bits 83 and up are copies of the sign, so bits
    // 52..83 of the sum are one signed 32-bit word z = sum >> 52 (a funnel shift of the top two
    // words), and the position of z's most significant bit that differs from its sign bit (bfind.s32;
    // -1 when there is none, for z = 0 or -1) is msb|sum| - 52, read for a negative sum from its one's
    // complement.
    const uint32_t z = (x2 << 12) | (x1 >> 20);
#ifdef __CUDA_ARCH__
    int f;
    asm("bfind.s32 %0, %1;" : "=r"(f) : "r"(z));
#else
    const uint32_t zm = static_cast<int32_t>(z) < 0 ? ~z : z;
    const int f = zm ? 31 - clz32(zm) : -1;
#endif
    const int b = f < 0 ? 0 : f;
    // round to a multiple of 2^b, nearest-even: add 2^(b-1) - 1 and the lowest kept bit, then cut
    const uint32_t mask = (1u << b) - 1u;
    const uint32_t hq = (mask >> 1) + ((x0 >> b) & (mask & 1u));
#ifdef __CUDA_ARCH__
    asm("add.cc.u32 %0, %0, %3;\n\taddc.cc.u32 %1, %1, 0;\n\taddc.u32 %2, %2, 0;"
        : "+r"(x0), "+r"(x1), "+r"(x2)
        : "r"(hq));
#else
    const uint64_t old = (static_cast<uint64_t>(x1) << 32) | x0, lo = old + hq;
    x2 += lo < old ? 1u : 0u;
    x0 = static_cast<uint32_t>(lo);
    x1 = static_cast<uint32_t>(lo >> 32);
#endif
    x0 &= ~mask;
}

// The binary64 encoding of x * 2^-62 for a value with at most 53 significant bits (a rounded sum)
// and |x| < 2^84. Zero gives +0, or -0 when negzero (a chain of -0 terms sums to -0).
PRK_HD uint64_t fx96_to_bits(uint32_t x0, uint32_t x1, uint32_t x2, bool negzero)
{
    const uint32_t sg = static_cast<uint32_t>(static_cast<int32_t>(x2) >> 31);
    uint64_t lo = ((static_cast<uint64_t>(x1) << 32) | x0) ^ ((static_cast<uint64_t>(sg) << 32) | sg);
    uint32_t hi = x2 ^ sg;
    lo += sg & 1u;  // + 1 completes the negation of a negative value
    hi += (sg & 1u) && lo == 0 ? 1u : 0u;
    if ((lo | hi) == 0) return negzero ? SIGN : 0ull;
    const int msb = hi ? 95 - clz32(hi) : 63 - clz64(lo);
    uint64_t m;  // the significand, leading bit at position 52
    if (msb >= 52) {
        const int sa = msb - 52;  // 0 .. 31: the bits below are zero (x is rounded)
        m = sa == 0 ? lo : ((static_cast<uint64_t>(hi) << (64 - sa)) | (lo >> sa));
    } else {
        m = lo << (52 - msb);
    }
    return (static_cast<uint64_t>(sg) << 63) | ((static_cast<uint64_t>(msb - FX96_F + 1022) << 52) + m);
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
