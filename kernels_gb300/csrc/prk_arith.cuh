// Per-point arithmetic of the stencil forms, shared by every kernel that evaluates a point.
//
//  fp64_point<P,R>    the reference expression in binary64: each product and each sum rounded
//                     once, in the generator's tap order (generate-cxx-stencil.py:15-38). The
//                     explicit __dmul_rn/__dadd_rn keep the compiler from contracting to FMA.
//  fp32c_point<P,R>   the compensated FP32 form: every PRK weight matrix is point-antisymmetric,
//                     W[-d] = -W[d], so the sum is sum over d>0 of w_d * (in[p+d] - in[p-d]). The
//                     difference of two FP32 integers below 2^24 is exact; w_d = hi + lo splits the
//                     weight to ~2^-48; the products' rounding errors come back through FMA and the
//                     sum's through TwoSum, giving a (hi, lo) pair accurate to ~2^-44 relative.
//  df_add             (hi, lo) += (s_hi, s_lo) for the two-float out accumulator.
#pragma once

#include "prk_fixed.cuh"
#include "prk_stencil.cuh"

namespace prk {

// The point-antisymmetry the FP32 form relies on, checked at compile time for every stencil.
__host__ __device__ constexpr bool antisymmetric(int pattern, int R)
{
    for (int dc = -R; dc <= R; ++dc)
        for (int dr = -R; dr <= R; ++dr)
            if (weight(pattern, R, dc, dr) != -weight(pattern, R, -dc, -dr)) return false;
    return true;
}
static_assert(antisymmetric(STAR, 1) && antisymmetric(STAR, 2) && antisymmetric(STAR, 3) && antisymmetric(STAR, 4) &&
                  antisymmetric(STAR, 5),
              "star weights must be antisymmetric");
static_assert(antisymmetric(GRID, 1) && antisymmetric(GRID, 2) && antisymmetric(GRID, 3) && antisymmetric(GRID, 4) &&
                  antisymmetric(GRID, 5),
              "grid weights must be antisymmetric");
static_assert(tap_count(STAR, 2) == 8 && tap_count(GRID, 2) == 20, "tap counts");

// s points at in(i,j) inside a row-major tile with leading dimension ld.
template <int P, int R, typename T>
__device__ __forceinline__ double fp64_point(const T* s, int ld)
{
    double acc = 0.0;
    bool first = true;
#pragma unroll
    for (int dc = -R; dc <= R; ++dc) {
#pragma unroll
        for (int dr = -R; dr <= R; ++dr) {
            const double w = weight(P, R, dc, dr);
            if (w != 0.0) {
                const double p = __dmul_rn(static_cast<double>(s[dr * ld + dc]), w);
                acc = first ? p : __dadd_rn(acc, p);
                first = false;
            }
        }
    }
    return acc;
}

// TwoSum (Knuth): a + b = s + e exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float ap = __fsub_rn(s, bp);
    e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}

// Fast2Sum (Dekker), valid when |a| >= |b| or a == 0.
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

template <int P, int R>
__device__ __forceinline__ void fp32c_point(const float* s, int ld, float& s_hi, float& s_lo)
{
    float hi = 0.0f, lo = 0.0f;
    bool first = true;
#pragma unroll
    for (int dc = -R; dc <= R; ++dc) {
#pragma unroll
        for (int dr = -R; dr <= R; ++dr) {
            const double w = weight(P, R, dc, dr);
            if (w > 0.0) {
                const float wh = split_hi(w), wl = split_lo(w);
                const float d = __fsub_rn(s[dr * ld + dc], s[-dr * ld - dc]);
                const float p = __fmul_rn(wh, d);
                float pe = __fmaf_rn(wh, d, -p);
                pe = __fmaf_rn(wl, d, pe);
                if (first) {
                    hi = p;
                    lo = pe;
                    first = false;
                } else {
                    float t, e;
                    two_sum(hi, p, t, e);
                    hi = t;
                    lo = __fadd_rn(lo, __fadd_rn(e, pe));
                }
            }
        }
    }
    s_hi = hi;
    s_lo = lo;
}

// fl(a + 1) without the binary64 pipe where that is exact (fx::inc_whole: positive whole numbers
// below 2^53); other values take the binary64 add.
__device__ __forceinline__ double inc_exact(double a)
{
    uint64_t r;
    if (fx::inc_whole(static_cast<uint64_t>(__double_as_longlong(a)), &r))
        return __longlong_as_double(static_cast<long long>(r));
    return __dadd_rn(a, 1.0);
}

// (o_hi, o_lo) += (s_hi, s_lo), renormalised so that |o_lo| <= ulp(o_hi)/2.
__device__ __forceinline__ void df_add(float& o_hi, float& o_lo, float s_hi, float s_lo)
{
    float t, e;
    two_sum(o_hi, s_hi, t, e);
    e = __fadd_rn(e, __fadd_rn(o_lo, s_lo));
    fast_two_sum(t, e, o_hi, o_lo);
}

// (o_hi, o_lo) += (s_hi, s_lo) without renormalising: o_hi takes the rounded sum of the high parts
// and o_lo collects its exact error and the low parts. A series of these (out held in registers
// across applications) ends with one fast_two_sum(o_hi, o_lo); o_lo stays a small multiple of the
// rounding errors, far inside FP32's range, so the pair keeps its accuracy.
__device__ __forceinline__ void df_add_lazy(float& o_hi, float& o_lo, float s_hi, float s_lo)
{
    float t, e;
    two_sum(o_hi, s_hi, t, e);
    o_hi = t;
    o_lo = __fadd_rn(o_lo, __fadd_rn(e, s_lo));
}

}  // namespace prk
