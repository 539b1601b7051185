// The TMA tile kernel, templated on pattern, radius, storage form and temporal depth.
//
// One CTA per TH x TW tile of the grid, as many resident per SM as shared memory allows. The elected
// thread issues two 2D TMA loads that complete on one mbarrier: the `in` tile with its halo and the
// `out` tile. The halo is R rows above and below and RA >= R columns either side, RA rounded up to
// 16 bytes so every TMA x coordinate is 16-byte aligned; the hardware zero-fills what lies outside
// the grid. The resident CTAs of an SM overlap one another's loads and evaluation. (A persistent
// variant with a ring of stages per CTA measured slower here: fewer warps per SM to evaluate each
// tile, and CTAs drifting apart in the raster order.)
//
// In a tile, lane l owns CPT adjacent columns (one 16-byte vector) and warp w owns the ROWS
// consecutive rows from w * ROWS, so that the rows of a thread share their vertical taps in
// registers. in_next and out go straight to HBM with 16-byte stores.
//
// Temporal depth STEPS: the tile applies STEPS consecutive applications before writing back.
// `in` evolves pointwise (in_{k+1} = in_k + 1, Cxx11/stencil-openmp.cc:208-218), so the copy in
// shared memory, halo included, is advanced in place with the same rounded +1 the reference
// applies, and the halo never grows. Every application reads the current `in` values and applies
// every tap. `out` stays in registers and is rounded after each application as the reference
// rounds it. HBM traffic per application drops by STEPS. STEPS = 0 takes the depth at run time
// (`depth`, any count): a whole run in one launch per tile, as the host-buffer path uses it on
// bands of rows.
//
// Evaluation modes:
//   FP64, strict   every point in the reference order with binary64 instructions (bit-exact)
//   FP64, exact    power-of-two stencils on a certified tile: integer evaluation with identical
//                  bits (prk_fixed.cuh), falling back to strict per tile
//   FP32C          paired antisymmetric differences from register row segments, summed per weight
//                  group, split weights, TwoSum, two-float out (prk_arith.cuh)
#pragma once

#include <cuda.h>

#include "prk_arith.cuh"
#include "prk_fixed.cuh"
#include "prk_internal.cuh"
#include "prk_ptx.cuh"

namespace prk {
namespace tile {

constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;

// Tile shape per storage form: TW columns (CPT per lane, one 16-byte vector) by TH rows (TH/8 per
// warp). TH is the tile-height variant the autotuner chooses between (32: 4 rows per thread; 64: 8).
template <int DT, int TH_ = 32>
struct Cfg;
template <int TH_>
struct Cfg<FP64, TH_> {
    using T = double;
    static constexpr int TW = 64, TH = TH_, CPT = 2, VEC = 2;
};
template <int TH_>
struct Cfg<FP32C, TH_> {
    using T = float;
    static constexpr int TW = 128, TH = TH_, CPT = 4, VEC = 4;
};
constexpr int TH_DEFAULT = 32;
constexpr int TH_TALL = 64;
// Deepest run-time depth for which the FP32 route holds: 15 * (2^20 + 65536) < 2^24.
constexpr int FP32_MAX_STEPS = 65536;

constexpr int SMEM_PER_SM = 228 * 1024;
constexpr int SMEM_PER_CTA_MAX = 227 * 1024;

template <int DT, int R, int TH_ = 32>
struct Geo {
    using C = Cfg<DT, TH_>;
    using T = typename C::T;
    static constexpr int RA = ((R + C::VEC - 1) / C::VEC) * C::VEC;  // halo columns, 16-byte multiple
    static constexpr int SW = C::TW + 2 * RA;                        // in-tile row length = TMA box x
    static constexpr int SH = C::TH + 2 * R;                         // in-tile rows = TMA box y
    static constexpr int IN_BYTES = SW * SH * static_cast<int>(sizeof(T));
    static constexpr int OUT_BYTES = C::TW * C::TH * 8;
    static constexpr int OUT_OFF = (IN_BYTES + 127) / 128 * 128;     // out tile
    static constexpr int RED_OFF = OUT_OFF + OUT_BYTES;              // per-warp words of the certification
    static constexpr int BAR_OFF = RED_OFF + WARPS * 8;
    static constexpr int SMEM = BAR_OFF + 8;
    static constexpr int CTAS_FIT = SMEM_PER_SM / (SMEM + 1024);     // 1 KB per CTA is reserved
    static constexpr int CTAS = CTAS_FIT > 8 ? 8 : CTAS_FIT;         // resident CTAs per SM
    static constexpr int ELEMS = SW * SH;
    static constexpr int ROWS = C::TH / WARPS;
    static_assert(SMEM <= SMEM_PER_CTA_MAX && CTAS >= 1, "the tile must fit in shared memory");
    static_assert(SW <= 256 && SH <= 256 && C::TW <= 256, "TMA box dimensions are at most 256");
    static_assert((SW * sizeof(T)) % 16 == 0, "TMA box rows must be 16-byte multiples");
    static_assert(C::TH % WARPS == 0 && C::TW == 32 * C::CPT, "thread layout");
};

// Everything a launch needs besides the template arguments.
struct Launch {
    CUtensorMap tm_in;
    CUtensorMap tm_out;
    int64_t n;
    void* in_next;
    void* out;
    unsigned* status;
    cudaStream_t stream;
    int depth;     // applications per launch for the run-time-depth kernels (STEPS = 0)
    int64_t row0;  // first array row of the launch's tiles
    int64_t rows;  // array rows covered from row0 (0: to the last row of the arrays)
    int64_t nr;    // rows the arrays hold (0: n, a whole grid); the tensor maps cover nr x n
    int64_t goff;  // grid row of the arrays' row 0
};

// ---------------------------------------------------------------------------------------------
// 16-byte vector access helpers

__device__ __forceinline__ void st_vec(double* p, const double (&v)[2])
{
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
}
__device__ __forceinline__ void st_vec(float* p, const float (&v)[4])
{
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}

// N consecutive floats from 16-byte-aligned shared memory.
template <int N>
__device__ __forceinline__ void ld_seg(const float* p, float (&v)[N])
{
    static_assert(N % 4 == 0, "segment is whole float4 vectors");
#pragma unroll
    for (int q = 0; q < N / 4; ++q) {
        const float4 t = reinterpret_cast<const float4*>(p)[q];
        v[4 * q] = t.x;
        v[4 * q + 1] = t.y;
        v[4 * q + 2] = t.z;
        v[4 * q + 3] = t.w;
    }
}

// N consecutive fixed-point words from 16-byte-aligned shared memory, narrowed to I.
template <int N, typename I>
__device__ __forceinline__ void ld_seg_i(const int64_t* p, I (&v)[N])
{
    static_assert(N % 2 == 0, "segment is whole 16-byte vectors");
#pragma unroll
    for (int q = 0; q < N / 2; ++q) {
        const longlong2 t = reinterpret_cast<const longlong2*>(p)[q];
        v[2 * q] = static_cast<I>(t.x);
        v[2 * q + 1] = static_cast<I>(t.y);
    }
}

// ---------------------------------------------------------------------------------------------
// FP32C: the stencil sums of CPT points of one row. s points at in(r, c0) in the smem tile.

// The taps of a PRK stencil share few distinct weights: star R has R (1/(2kR) on the k-th ring of
// the cross), grid R has 2R (the sides and the diagonal of each ring). Group g collects the paired
// differences whose weight is +-c_g: D_g = sum of sign * (in[p+d] - in[p-d]). Every tap's two values
// are read and differenced; the sums within a group are exact for integer fields (they stay below
// 2^24), and the weights then enter through NG compensated products instead of one per tap.
template <int P, int R>
__host__ __device__ constexpr int group_count() { return P == STAR ? R : 2 * R; }

// Group of the positive tap (dc, dr) (dr > 0, or dr == 0 and dc > 0) and the sign of its weight.
template <int P, int R>
__host__ __device__ constexpr int group_of(int dc, int dr)
{
    const int adc = dc > 0 ? dc : -dc, adr = dr > 0 ? dr : -dr;
    const int m = adc > adr ? adc : adr;
    if (P == STAR) return m - 1;
    return (adc == m && adr == m) ? R + m - 1 : m - 1;  // diagonal of ring m, else its sides
}

// |weight| of group g, as a (hi, lo) float pair.
template <int P, int R>
__host__ __device__ constexpr double group_weight(int g)
{
    if (P == STAR) return weight(STAR, R, 0, g + 1);
    return g < R ? weight(GRID, R, 0, g + 1) : weight(GRID, R, g - R + 1, g - R + 1);
}

// Every positive tap's |weight| is its group's weight (checked at compile time for all stencils).
template <int P, int R>
__host__ __device__ constexpr bool groups_ok()
{
    for (int dr = 0; dr <= R; ++dr)
        for (int dc = -R; dc <= R; ++dc) {
            if (dr == 0 && dc <= 0) continue;
            const double w = weight(P, R, dc, dr);
            if (w != 0.0 && (w > 0 ? w : -w) != group_weight<P, R>(group_of<P, R>(dc, dr))) return false;
        }
    return true;
}
static_assert(groups_ok<STAR, 1>() && groups_ok<STAR, 2>() && groups_ok<STAR, 3>() && groups_ok<STAR, 4>() &&
                  groups_ok<STAR, 5>() && groups_ok<GRID, 1>() && groups_ok<GRID, 2>() && groups_ok<GRID, 3>() &&
                  groups_ok<GRID, 4>() && groups_ok<GRID, 5>(),
              "weight groups");

template <int P, int R, int CPT, int RA>
__device__ __forceinline__ void fp32c_points(const float* s, int ld, float (&sh)[CPT], float (&sl)[CPT])
{
    constexpr int SEG = CPT + 2 * RA;
    constexpr int NG = group_count<P, R>();
    float D[NG][CPT];
    bool seen[NG];  // a group's sum starts from its first difference (known once the loops unroll)
#pragma unroll
    for (int g = 0; g < NG; ++g) {
        seen[g] = false;
#pragma unroll
        for (int k = 0; k < CPT; ++k) D[g][k] = 0.0f;
    }
    {
        float m0[SEG];
        ld_seg<SEG>(s - RA, m0);
#pragma unroll
        for (int dc = 1; dc <= R; ++dc) {
            constexpr int dr = 0;
            const int g = group_of<P, R>(dc, dr);
#pragma unroll
            for (int k = 0; k < CPT; ++k) {
                const float d = __fsub_rn(m0[k + RA + dc], m0[k + RA - dc]);
                D[g][k] = seen[g] ? __fadd_rn(D[g][k], d) : d;
            }
            seen[g] = true;
        }
    }
#pragma unroll
    for (int dr = 1; dr <= R; ++dr) {
        if constexpr (P == STAR) {
            float up[CPT], dn[CPT];
            ld_seg<CPT>(s + dr * ld, up);
            ld_seg<CPT>(s - dr * ld, dn);
            const int g = group_of<P, R>(0, dr);
#pragma unroll
            for (int k = 0; k < CPT; ++k) {
                const float d = __fsub_rn(up[k], dn[k]);
                D[g][k] = seen[g] ? __fadd_rn(D[g][k], d) : d;
            }
            seen[g] = true;
        } else {
            float up[SEG], dn[SEG];
            ld_seg<SEG>(s + dr * ld - RA, up);
            ld_seg<SEG>(s - dr * ld - RA, dn);
#pragma unroll
            for (int dc = -R; dc <= R; ++dc) {
                const int sg = weight_sign(P, R, dc, dr);
                if (sg != 0) {
                    const int g = group_of<P, R>(dc, dr);
#pragma unroll
                    for (int k = 0; k < CPT; ++k) {
                        const float d = __fsub_rn(up[k + RA + dc], dn[k + RA - dc]);
                        if (seen[g])
                            D[g][k] = sg > 0 ? __fadd_rn(D[g][k], d) : __fsub_rn(D[g][k], d);
                        else
                            D[g][k] = sg > 0 ? d : -d;
                    }
                    seen[g] = true;
                }
            }
        }
    }
    // S = sum over groups of c_g * D_g: products with split weights and their errors through FMA,
    // the sum through TwoSum, giving (hi, lo)
#pragma unroll
    for (int g = 0; g < NG; ++g) {
        const double w = group_weight<P, R>(g);
        const float wh = split_hi(w), wl = split_lo(w);
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            const float p = __fmul_rn(wh, D[g][k]);
            float pe = __fmaf_rn(wh, D[g][k], -p);
            pe = __fmaf_rn(wl, D[g][k], pe);
            if (g == 0) {
                sh[k] = p;
                sl[k] = pe;
            } else {
                float t, e;
                two_sum(sh[k], p, t, e);
                sh[k] = t;
                sl[k] = __fadd_rn(sl[k], __fadd_rn(e, pe));
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// FP64 exact route: integer coefficients c = w * 2^shift of a power-of-two stencil.

template <int P, int R>
__device__ __forceinline__ constexpr int coef(int dc, int dr)
{
    const int d = weight_den(P, R, dc, dr);
    return d == 0 ? 0 : weight_sign(P, R, dc, dr) * ((1 << pow2_shift(P, R)) / d);
}

// sum of c * (V[p+d] - V[p-d]) over the positive taps for CPT points of a row; v points at V(r, c0).
template <int P, int R, int CPT, int RA, typename I>
__device__ __forceinline__ void fx_points(const int64_t* v, int ld, I (&S)[CPT])
{
    constexpr int SEG = CPT + 2 * RA;
#pragma unroll
    for (int k = 0; k < CPT; ++k) S[k] = 0;
    {
        I m0[SEG];
        ld_seg_i<SEG>(v - RA, m0);
#pragma unroll
        for (int dc = 1; dc <= R; ++dc) {
            const int cc = coef<P, R>(dc, 0);
#pragma unroll
            for (int k = 0; k < CPT; ++k) S[k] += static_cast<I>(cc) * (m0[k + RA + dc] - m0[k + RA - dc]);
        }
    }
#pragma unroll
    for (int dr = 1; dr <= R; ++dr) {
        if constexpr (P == STAR) {
            I up[CPT], dn[CPT];
            ld_seg_i<CPT>(v + dr * ld, up);
            ld_seg_i<CPT>(v - dr * ld, dn);
            const int cc = coef<P, R>(0, dr);
#pragma unroll
            for (int k = 0; k < CPT; ++k) S[k] += static_cast<I>(cc) * (up[k] - dn[k]);
        } else {
            I up[SEG], dn[SEG];
            ld_seg_i<SEG>(v + dr * ld - RA, up);
            ld_seg_i<SEG>(v - dr * ld - RA, dn);
#pragma unroll
            for (int dc = -R; dc <= R; ++dc) {
                const int cc = coef<P, R>(dc, dr);
                if (cc != 0) {
#pragma unroll
                    for (int k = 0; k < CPT; ++k) S[k] += static_cast<I>(cc) * (up[k + RA + dc] - dn[k + RA - dc]);
                }
            }
        }
    }
}

// N consecutive floats from 8-byte-aligned shared memory (float2 loads).
template <int N>
__device__ __forceinline__ void ld_seg2(const float* p, float (&v)[N])
{
    static_assert(N % 2 == 0, "segment is whole float2 vectors");
#pragma unroll
    for (int q = 0; q < N / 2; ++q) {
        const float2 t = reinterpret_cast<const float2*>(p)[q];
        v[2 * q] = t.x;
        v[2 * q + 1] = t.y;
    }
}

// The integer route in FP32: every value of the tile is an integer below 2^20, so the differences,
// the products by the small integer coefficients and every partial sum are integers below 2^24 and
// FP32 arithmetic is exact. Sum of c * (V[p+d] - V[p-d]) for CPT points; v points at V(r, c0).
template <int P, int R, int CPT, int RA>
__device__ __forceinline__ void fexact_points(const float* v, int ld, float (&S)[CPT])
{
    constexpr int SEG = CPT + 2 * RA;
#pragma unroll
    for (int k = 0; k < CPT; ++k) S[k] = 0.0f;
    {
        float m0[SEG];
        ld_seg2<SEG>(v - RA, m0);
#pragma unroll
        for (int dc = 1; dc <= R; ++dc) {
            const float cc = static_cast<float>(coef<P, R>(dc, 0));
#pragma unroll
            for (int k = 0; k < CPT; ++k) S[k] = __fmaf_rn(cc, __fsub_rn(m0[k + RA + dc], m0[k + RA - dc]), S[k]);
        }
    }
#pragma unroll
    for (int dr = 1; dr <= R; ++dr) {
        if constexpr (P == STAR) {
            float up[CPT], dn[CPT];
            ld_seg2<CPT>(v + dr * ld, up);
            ld_seg2<CPT>(v - dr * ld, dn);
            const float cc = static_cast<float>(coef<P, R>(0, dr));
#pragma unroll
            for (int k = 0; k < CPT; ++k) S[k] = __fmaf_rn(cc, __fsub_rn(up[k], dn[k]), S[k]);
        } else {
            float up[SEG], dn[SEG];
            ld_seg2<SEG>(v + dr * ld - RA, up);
            ld_seg2<SEG>(v - dr * ld - RA, dn);
#pragma unroll
            for (int dc = -R; dc <= R; ++dc) {
                const int c = coef<P, R>(dc, dr);
                if (c != 0) {
#pragma unroll
                    for (int k = 0; k < CPT; ++k)
                        S[k] = __fmaf_rn(static_cast<float>(c), __fsub_rn(up[k + RA + dc], dn[k + RA - dc]), S[k]);
                }
            }
        }
    }
}

// fexact_points for the ROWS consecutive rows of a thread at once: S[rr] for the CPT points of row
// r0 + rr, v pointing at V(r0, c0); own[rr] gets the values of those points. Every row segment
// (star: every column strip) is read from shared memory once and serves every row it is a tap of.
// The arithmetic is exact, so the order of the terms does not matter.
template <int P, int R, int CPT, int ROWS, int RA>
__device__ __forceinline__ void fexact_rows(const float* v, int ld, float (&S)[ROWS][CPT], float (&own)[ROWS][CPT])
{
    constexpr int SEG = CPT + 2 * RA;
    constexpr int NR = ROWS + 2 * R;  // rows r0 - R .. r0 + ROWS - 1 + R
    if constexpr (P == STAR) {
        float col[NR][CPT];
#pragma unroll
        for (int q = 0; q < NR; ++q)
            if (q < R || q >= R + ROWS) ld_seg2<CPT>(v + (q - R) * ld, col[q]);
#pragma unroll
        for (int rr = 0; rr < ROWS; ++rr) {
            float m[SEG];
            ld_seg2<SEG>(v + rr * ld - RA, m);
#pragma unroll
            for (int k = 0; k < CPT; ++k) {
                col[rr + R][k] = m[k + RA];
                own[rr][k] = m[k + RA];
                S[rr][k] = 0.0f;
            }
#pragma unroll
            for (int dc = 1; dc <= R; ++dc) {
                const float cc = static_cast<float>(coef<P, R>(dc, 0));
#pragma unroll
                for (int k = 0; k < CPT; ++k)
                    S[rr][k] = __fmaf_rn(cc, __fsub_rn(m[k + RA + dc], m[k + RA - dc]), S[rr][k]);
            }
        }
#pragma unroll
        for (int rr = 0; rr < ROWS; ++rr)
#pragma unroll
            for (int dr = 1; dr <= R; ++dr) {
                const float cc = static_cast<float>(coef<P, R>(0, dr));
#pragma unroll
                for (int k = 0; k < CPT; ++k)
                    S[rr][k] = __fmaf_rn(cc, __fsub_rn(col[rr + R + dr][k], col[rr + R - dr][k]), S[rr][k]);
            }
    } else {
        float seg[NR][SEG];
#pragma unroll
        for (int q = 0; q < NR; ++q) ld_seg2<SEG>(v + (q - R) * ld - RA, seg[q]);
#pragma unroll
        for (int rr = 0; rr < ROWS; ++rr) {
#pragma unroll
            for (int k = 0; k < CPT; ++k) {
                S[rr][k] = 0.0f;
                own[rr][k] = seg[rr + R][k + RA];
            }
#pragma unroll
            for (int dr = 0; dr <= R; ++dr)
#pragma unroll
                for (int dc = -R; dc <= R; ++dc) {
                    if (dr == 0 && dc <= 0) continue;
                    const int c = coef<P, R>(dc, dr);
                    if (c != 0) {
#pragma unroll
                        for (int k = 0; k < CPT; ++k)
                            S[rr][k] = __fmaf_rn(static_cast<float>(c),
                                                 __fsub_rn(seg[rr + R + dr][k + RA + dc], seg[rr + R - dr][k + RA - dc]),
                                                 S[rr][k]);
                    }
                }
        }
    }
}

// binary64 encoding of f * 2^adj for an integer-valued f (|f| < 2^24): exponent rebias and a
// mantissa shift, no conversion instruction (those run on the binary64 pipe).
__device__ __forceinline__ uint64_t f2d(float f, int adj)
{
    const uint32_t u = __float_as_uint(f);
    const uint64_t mag = u & 0x7FFFFFFFu;
    const uint64_t d = (static_cast<uint64_t>(u & 0x80000000u) << 32) |
                       ((mag + (static_cast<uint64_t>(896 + adj) << 23)) << 29);
    return mag == 0 ? 0ull : d;
}

// binary64 encoding of x * 2^unit for a 32-bit x (exact).
__device__ __forceinline__ uint64_t from_fixed32(int32_t x, int unit)
{
    if (x == 0) return 0;
    const uint64_t s = x < 0 ? fx::SIGN : 0;
    const uint32_t a = x < 0 ? static_cast<uint32_t>(-x) : static_cast<uint32_t>(x);
    const int msb = 31 - __clz(a);
    const uint64_t m = static_cast<uint64_t>(a) << (52 - msb);
    return s | ((static_cast<uint64_t>(msb + unit + 1022) << 52) + m);
}

// out = V * 2^-shift for an integer V with |V| < 2^21, read from the binary64 encoding (+-0 give 0);
// false for any other value. With M the 53-bit significand, V = M >> (k + 32) for
// k = 1043 - shift - (biased exponent), an integer below 2^21 exactly when 0 <= k <= 20 and the
// k + 32 bits shifted out are zero. Subnormals, infinities and NaNs fall outside that range of k.
__device__ __forceinline__ bool out_units(uint64_t b, int shift, int32_t& V)
{
    const uint32_t hi = static_cast<uint32_t>(b >> 32), lo = static_cast<uint32_t>(b);
    const uint32_t mag = hi & 0x7FFFFFFFu;
    const int k = 1043 - shift - static_cast<int>(mag >> 20);
    const uint32_t m = (mag & 0xFFFFFu) | 0x100000u;
    const bool zero = (mag | lo) == 0u;
    const bool ok = zero || (lo == 0u && k >= 0 && k <= 20 && (m & ((1u << (k & 31)) - 1u)) == 0u);
    const int32_t a = static_cast<int32_t>(m >> (k & 31));
    V = zero ? 0 : ((hi >> 31) ? -a : a);
    return ok;
}

__device__ __forceinline__ uint64_t from_fixed_any(int64_t x, int unit) { return fx::from_fixed(x, unit); }
__device__ __forceinline__ uint64_t from_fixed_any(int32_t x, int unit) { return from_fixed32(x, unit); }

__device__ __forceinline__ double as_dbl(uint64_t b) { return __longlong_as_double(static_cast<long long>(b)); }
__device__ __forceinline__ uint64_t as_bits(double d) { return static_cast<uint64_t>(__double_as_longlong(d)); }

// in += 1 over the whole staged tile, halo included, as 16-byte vectors (the tile starts at the
// 128-byte aligned stage and its element count is a multiple of four): FP32 values (the FP32 route
// and FP32C), integers in fixed-point units (one = 1.0 in those units) or binary64 values.
template <int ELEMS>
__device__ __forceinline__ void advance_f32(float* p)
{
    constexpr int NV = ELEMS / 4;
#pragma unroll
    for (int q = 0; q < (NV + THREADS - 1) / THREADS; ++q) {
        const int idx = threadIdx.x + q * THREADS;
        if (NV % THREADS == 0 || idx < NV) {
            float4 v = reinterpret_cast<float4*>(p)[idx];
            v.x = __fadd_rn(v.x, 1.0f);
            v.y = __fadd_rn(v.y, 1.0f);
            v.z = __fadd_rn(v.z, 1.0f);
            v.w = __fadd_rn(v.w, 1.0f);
            reinterpret_cast<float4*>(p)[idx] = v;
        }
    }
}

// dst = src + 1 over the halo of a staged FP32 tile only (the R rows above and below, the RA
// columns either side): the interior points are advanced by the threads that own them. Rows as
// 16-byte vectors, side columns as 8-byte pairs.
template <int SW, int SH, int R, int RA>
__device__ __forceinline__ void advance_halo_f32(const float* src, float* dst)
{
    static_assert(SW % 4 == 0 && RA % 2 == 0, "halo vectors");
    constexpr int ROWV = SW / 4;               // 16-byte vectors in a row
    constexpr int NROW = 2 * R * ROWV;         // top and bottom halo rows
    constexpr int PER_SIDE = RA / 2;           // 8-byte pairs per side of a row
    constexpr int NSIDE = (SH - 2 * R) * 2 * PER_SIDE;
#pragma unroll
    for (int q = 0; q < (NROW + NSIDE + THREADS - 1) / THREADS; ++q) {
        const int h = threadIdx.x + q * THREADS;
        if (h < NROW) {
            const int r = h / ROWV, v = h - r * ROWV;
            const int row = r < R ? r : SH - 2 * R + r;  // rows 0..R-1, then SH-R..SH-1
            float4 x = reinterpret_cast<const float4*>(src + row * SW)[v];
            x.x = __fadd_rn(x.x, 1.0f);
            x.y = __fadd_rn(x.y, 1.0f);
            x.z = __fadd_rn(x.z, 1.0f);
            x.w = __fadd_rn(x.w, 1.0f);
            reinterpret_cast<float4*>(dst + row * SW)[v] = x;
        } else if (h < NROW + NSIDE) {
            const int i = h - NROW;
            const int row = R + i / (2 * PER_SIDE), p = i - (i / (2 * PER_SIDE)) * (2 * PER_SIDE);
            const int col = p < PER_SIDE ? 2 * p : SW - RA + 2 * (p - PER_SIDE);
            float2 x = *reinterpret_cast<const float2*>(src + row * SW + col);
            x.x = __fadd_rn(x.x, 1.0f);
            x.y = __fadd_rn(x.y, 1.0f);
            *reinterpret_cast<float2*>(dst + row * SW + col) = x;
        }
    }
}

template <int ELEMS>
__device__ __forceinline__ void advance_i64(int64_t* p, int64_t one)
{
    constexpr int NV = ELEMS / 2;
#pragma unroll
    for (int q = 0; q < (NV + THREADS - 1) / THREADS; ++q) {
        const int idx = threadIdx.x + q * THREADS;
        if (NV % THREADS == 0 || idx < NV) {
            longlong2 v = reinterpret_cast<longlong2*>(p)[idx];
            v.x += one;
            v.y += one;
            reinterpret_cast<longlong2*>(p)[idx] = v;
        }
    }
}

template <int ELEMS>
__device__ __forceinline__ void advance_f64(double* p)
{
    constexpr int NV = ELEMS / 2;
#pragma unroll
    for (int q = 0; q < (NV + THREADS - 1) / THREADS; ++q) {
        const int idx = threadIdx.x + q * THREADS;
        if (NV % THREADS == 0 || idx < NV) {
            double2 v = reinterpret_cast<double2*>(p)[idx];
            v.x = inc_exact(v.x);
            v.y = inc_exact(v.y);
            reinterpret_cast<double2*>(p)[idx] = v;
        }
    }
}

// binary64 encoding of a constexpr double (normal or zero), by exact scaling by powers of two
// (C++17 has no bit_cast in constant expressions).
__host__ __device__ constexpr uint64_t encode(double w)
{
    if (w == 0.0) return 0;
    uint64_t sign = 0;
    if (w < 0) {
        sign = fx::SIGN;
        w = -w;
    }
    int e = 0;
    while (w >= 2.0) {
        w /= 2.0;
        ++e;
    }
    while (w < 1.0) {
        w *= 2.0;
        --e;
    }
    const uint64_t frac = static_cast<uint64_t>((w - 1.0) * 4503599627370496.0);  // exact: 52 bits
    return sign | (static_cast<uint64_t>(e + 1023) << 52) | frac;
}
static_assert(encode(1.0) == 0x3FF0000000000000ull && encode(-0.125) == 0xBFC0000000000000ull &&
                  encode(1.0 / 6.0) == 0x3FC5555555555555ull,
              "constexpr binary64 encoding");

// The taps of a stencil in the generator's order (column offset outer, row offset inner, zero
// weights left out), with their offsets in a tile of row length LD and their weights split for
// fx::mul_whole20_split: the significand's low 32 bits, its high 21 bits with the hidden bit, and
// the sign and exponent field of the encoding's high word. One 16-byte entry per tap.
template <int P, int R, int LD>
struct TapTable {
    struct alignas(16) Tap {
        int off;
        uint32_t w1, w2, hib;
    } tap[tap_count(P, R)];
};

template <int P, int R, int LD>
constexpr TapTable<P, R, LD> make_taps()
{
    TapTable<P, R, LD> t{};
    int k = 0;
    for (int dc = -R; dc <= R; ++dc)
        for (int dr = -R; dr <= R; ++dr) {
            const double w = weight(P, R, dc, dr);
            if (w != 0.0) {
                const uint64_t wb = encode(w);
                t.tap[k].off = dr * LD + dc;
                t.tap[k].w1 = static_cast<uint32_t>(wb);
                t.tap[k].w2 = static_cast<uint32_t>((wb >> 32) & 0xFFFFFu) | 0x100000u;
                t.tap[k].hib = static_cast<uint32_t>(wb >> 32) & 0xFFF00000u;
                ++k;
            }
        }
    return t;
}

template <int P, int R, int LD>
__constant__ TapTable<P, R, LD> c_taps = make_taps<P, R, LD>();

// fp64_point for CPT adjacent points of a tile of whole numbers |v| < 2^20 held as int32: every
// product comes from fx::mul_whole20_split on the integer pipes (the same bits as __dmul_rn), every sum is
// the same binary64 add in the same order, so the binary64 pipe issues one instruction per tap
// instead of two. The taps come from constant memory in a loop, which keeps the code small.
template <int P, int R, int LD, int CPT>
__device__ __forceinline__ void fp64_points_whole(const int32_t* s, double (&acc)[CPT])
{
    constexpr int N = tap_count(P, R);
    const auto& T = c_taps<P, R, LD>;
    {
        const auto tp = T.tap[0];
#pragma unroll
        for (int k = 0; k < CPT; ++k)
            acc[k] = __longlong_as_double(
                static_cast<long long>(fx::mul_whole20_split(tp.w1, tp.w2, tp.hib, s[tp.off + k])));
    }
#pragma unroll 2
    for (int t = 1; t < N; ++t) {
        const auto tp = T.tap[t];
#pragma unroll
        for (int k = 0; k < CPT; ++k)
            acc[k] = __dadd_rn(acc[k], __longlong_as_double(static_cast<long long>(
                                           fx::mul_whole20_split(tp.w1, tp.w2, tp.hib, s[tp.off + k]))));
    }
}

// in += 1 over a staged tile of int32 whole numbers, as 16-byte vectors.
template <int ELEMS>
__device__ __forceinline__ void advance_i32(int32_t* p)
{
    constexpr int NV = ELEMS / 4;
#pragma unroll
    for (int q = 0; q < (NV + THREADS - 1) / THREADS; ++q) {
        const int idx = threadIdx.x + q * THREADS;
        if (NV % THREADS == 0 || idx < NV) {
            int4 v = reinterpret_cast<int4*>(p)[idx];
            v.x += 1;
            v.y += 1;
            v.z += 1;
            v.w += 1;
            reinterpret_cast<int4*>(p)[idx] = v;
        }
    }
}

// Where process_tile finds `out`: the out tile loaded into shared memory next to `in` (TMA path), or
// HBM, read in the evaluation row by row (batched path) or with every row's words requested before
// the first row is evaluated (plain-staged path; used for the FP64 power-of-two stencils at one
// application, where it measured faster, and like OUT_HBM otherwise).
constexpr int OUT_SMEM = 0, OUT_HBM = 1, OUT_HBM_AHEAD = 2;

// ---------------------------------------------------------------------------------------------
// FP64 stencils whose weights are not powers of two, on whole-number tiles of small range: the
// table route.
//
// Every product and every partial sum of the reference's chain rounds, and GB300 issues binary64
// adds at a small fraction of its integer rate, so the route moves work off the binary64 pipe
// without changing a bit:
//  - Products from a table. A tile whose values all lie in [base, base + TBL_L) takes each product
//    fl(|w| * v) from a shared-memory table of every weight group and every such v, built once per
//    tile with fx::mul_whole20 (the weight's sign enters as an add or a subtract). Every tap still
//    reads its own in value, and indexes the table with it.
//  - The first fixed_taps() adds of each point's chain run in 96-bit fixed point on the integer
//    pipes (fx::fx96_acc_round: the exact sum rounded to 53 bits, nearest-even, the binary64 add's
//    result bit for bit on these values), the rest and the add into out on the binary64 pipe.
// Lane l evaluates columns l and l + 32 of its warp's rows, so a warp's table reads are consecutive
// entries; the results go into the shared-memory out tile, which the stores then read in their own
// layout. Applications of a multi-application launch write in + 1 to the other half of the stage
// (the int32 tile takes half of it), and the table is rebuilt at a new base when the values outgrow
// it.

constexpr int TBL_L = 128;  // consecutive values one product table covers

// The tables follow the TMA kernel's own shared memory (16-byte aligned).
template <int DT, int R, int TH_>
__host__ __device__ constexpr int table_offset()
{
    return (Geo<DT, R, TH_>::SMEM + 15) / 16 * 16;
}

template <int P, int R>
struct StrictTaps {
    int dc[tap_count(P, R)], dr[tap_count(P, R)], g[tap_count(P, R)], neg[tap_count(P, R)];
};

// The taps in the generator's order (column offset outer, row offset inner, zeros left out), each
// with its weight group and sign.
template <int P, int R>
constexpr StrictTaps<P, R> make_strict_taps()
{
    StrictTaps<P, R> t{};
    int k = 0;
    for (int dc = -R; dc <= R; ++dc)
        for (int dr = -R; dr <= R; ++dr) {
            const double w = weight(P, R, dc, dr);
            if (w != 0.0) {
                t.dc[k] = dc;
                t.dr[k] = dr;
                t.g[k] = group_of<P, R>(dc, dr);
                t.neg[k] = w < 0.0 ? 1 : 0;
                ++k;
            }
        }
    return t;
}

// Every tap's |weight| is its group's (checked for the stencils the route serves).
template <int P, int R>
constexpr bool strict_taps_ok()
{
    constexpr StrictTaps<P, R> t = make_strict_taps<P, R>();
    for (int k = 0; k < tap_count(P, R); ++k) {
        const double w = weight(P, R, t.dc[k], t.dr[k]);
        if ((w < 0.0 ? -w : w) != group_weight<P, R>(t.g[k])) return false;
    }
    return true;
}
static_assert(strict_taps_ok<STAR, 3>() && strict_taps_ok<STAR, 4>() && strict_taps_ok<STAR, 5>() &&
                  strict_taps_ok<GRID, 2>() && strict_taps_ok<GRID, 3>() && strict_taps_ok<GRID, 4>() &&
                  strict_taps_ok<GRID, 5>(),
              "strict tap groups");

// Sixteenths of each chain that run in fixed point (the rest stays on the binary64 pipe), per stencil
// and form (ONE: one application per launch; else several, where the tile's load is shared by the
// applications and the integer pipes take more of the chain), as measured best at n=16384 among 9 to
// 15 sixteenths (GFLOP/s, best against the next best):
//  - one application: star R=3, 4 11/16 (2150 against 2098 at 12/16 for R=4), R=5 12/16 (2066
//    against 2031 at 13/16); grid R=2 11/16 (2745 against 2704 at 12/16), R=3 12/16 (2870 against
//    2859 at 11/16), R=4 13/16 (2728 against 2721 at 14/16), R=5 15/16 (2656 against 2621 at 13/16);
//  - several (whole runs of 20): star R=3 14/16 (2777 against 2714 at 12/16), R=4, 5 13/16 (2930
//    against 2898 at 14/16 for R=5); grid R=2, 3 12/16 (3616 against 3557 at 13/16 for R=2), R=4
//    14/16 (3444 against 3419 at 13/16), R=5 13/16 (3222 against 3148 at 12/16).
template <int P, int R, bool ONE>
__host__ __device__ constexpr int fixed_sixteenths()
{
    if (P == STAR) {
        if (ONE) return R == 5 ? 12 : 11;
        return R == 3 ? 14 : 13;
    }
    if (ONE) return R == 2 ? 11 : (R == 3 ? 12 : (R == 4 ? 13 : 15));
    return R <= 3 ? 12 : (R == 4 ? 14 : 13);
}

// Taps of each chain whose adds run in fixed point (at least the first).
template <int P, int R, bool ONE>
__host__ __device__ constexpr int fixed_taps()
{
    const int k = tap_count(P, R) * fixed_sixteenths<P, R, ONE>() / 16;
    return k < 1 ? 1 : (k > tap_count(P, R) ? tap_count(P, R) : k);
}

// True when a positive weight lies among the fixed taps: then the fixed part never sums to -0 (a
// rounded sum is -0 only when every term is -0, and w * v with w > 0 is never -0).
template <int P, int R, bool ONE>
constexpr bool fixed_prefix_has_positive()
{
    constexpr StrictTaps<P, R> t = make_strict_taps<P, R>();
    for (int k = 0; k < fixed_taps<P, R, ONE>(); ++k)
        if (!t.neg[k]) return true;
    return false;
}

template <int P, int R, int DT>
__host__ __device__ constexpr bool table_route()
{
    return DT == FP64 && !pow2_weights(P, R);
}

// Shared memory of the tables: per weight group TBL_L binary64 products and TBL_L fixed-point images.
template <int P, int R, int DT>
__host__ __device__ constexpr int table_bytes()
{
    return table_route<P, R, DT>() ? group_count<P, R>() * TBL_L * (8 + 16) : 0;
}

// Dynamic shared memory of the TMA kernel: its tile stages, and the tables where the route applies.
template <int P, int R, int DT, int TH_>
__host__ __device__ constexpr int tile_smem()
{
    return table_offset<DT, R, TH_>() + table_bytes<P, R, DT>();
}

// Fill the tables for the values [base, base + TBL_L): T64[g * TBL_L + u] = fl(|w_g| * (base + u))
// and T96 its fixed-point image. Values at or beyond 2^20 in magnitude (never read) get 0.
template <int P, int R>
__device__ __forceinline__ void build_tables(uint64_t* T64, uint4* T96, int base)
{
    constexpr int NG = group_count<P, R>();
#pragma unroll
    for (int g = 0; g < NG; ++g) {
        const uint64_t wb = encode(group_weight<P, R>(g));
        for (int u = threadIdx.x; u < TBL_L; u += THREADS) {
            const int v = base + u;
            const uint64_t p = (v > -(1 << 20) && v < (1 << 20)) ? fx::mul_whole20(wb, v) : 0ull;
            uint32_t x0, x1, x2;
            fx::fx96_from_bits(p, x0, x1, x2);
            T64[g * TBL_L + u] = p;
            T96[g * TBL_L + u] = make_uint4(x0, x1, x2, 0u);
        }
    }
}

// x = fl(x + s * p) in fixed point, s the tap's sign.
__device__ __forceinline__ void fx96_tap(uint32_t (&x)[3], const uint4& p, int neg)
{
    if (neg)
        fx::fx96_acc_round<true>(x[0], x[1], x[2], p.x, p.y, p.z);
    else
        fx::fx96_acc_round<false>(x[0], x[1], x[2], p.x, p.y, p.z);
}

// Where a row of the table route's points lies: a row whose points are all outside the interior or
// past row_end is skipped (row-uniform); a column outside the interior is computed and dropped.
__device__ __forceinline__ bool table_row_active(bool has_out, int64_t gi, int64_t gg, int64_t row_end, int64_t n, int R)
{
    return has_out && gi < row_end && gg >= R && gg < n - R;
}

// The chain S of the points (r, c) and (r, c + 32): the reference's sum of fl(w * v) over the taps in
// the generator's order, the adds of its first fixed_taps<P, R, ONE>() taps in fixed point. sp points
// at the int32 tile's (r, c) (row stride SW); the tables cover [base, base + TBL_L).
template <int P, int R, int SW, bool ONE>
__device__ __forceinline__ void table_chain(const int32_t* sp, const uint64_t* T64, const uint4* T96, int base,
                                            double (&d)[2])
{
    constexpr StrictTaps<P, R> TP = make_strict_taps<P, R>();
    constexpr int N = tap_count(P, R), KF = fixed_taps<P, R, ONE>();
    constexpr bool POS = fixed_prefix_has_positive<P, R, ONE>();
    uint32_t x[2][3];
    int anyv[2] = {0, 0};
#pragma unroll
    for (int t = 0; t < KF; ++t) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int v = sp[TP.dr[t] * SW + TP.dc[t] + 32 * h];
            if (!POS) anyv[h] |= v;
            const uint4 p = T96[TP.g[t] * TBL_L + (v - base)];
            if (t == 0) {
                if (TP.neg[t]) {  // x = -p, the 96-bit two's-complement negation
                    x[h][0] = ~p.x + 1u;
                    x[h][1] = ~p.y + (p.x == 0u ? 1u : 0u);
                    x[h][2] = ~p.z + ((p.x | p.y) == 0u ? 1u : 0u);
                } else {
                    x[h][0] = p.x;
                    x[h][1] = p.y;
                    x[h][2] = p.z;
                }
            } else {
                fx96_tap(x[h], p, TP.neg[t]);
            }
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) d[h] = as_dbl(fx::fx96_to_bits(x[h][0], x[h][1], x[h][2], !POS && anyv[h] == 0));
#pragma unroll
    for (int t = KF; t < N; ++t) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int v = sp[TP.dr[t] * SW + TP.dc[t] + 32 * h];
            const double p = as_dbl(T64[TP.g[t] * TBL_L + (v - base)]);
            d[h] = TP.neg[t] ? __dsub_rn(d[h], p) : __dadd_rn(d[h], p);
        }
    }
}

// Bytes of the shared-memory out area the table route needs besides its tables in kernels that keep
// out in HBM (one FP64 tile of out words; the TMA kernel updates its out tile instead).
__host__ __device__ constexpr int table_out_bytes() { return Cfg<FP64>::TW * Cfg<FP64>::TH * 8; }

// dst = src + 1 over a whole int32 tile, halo included, as 16-byte vectors.
template <int ELEMS>
__device__ __forceinline__ void advance_i32_to(const int32_t* src, int32_t* dst)
{
    constexpr int NV = ELEMS / 4;
#pragma unroll
    for (int q = 0; q < (NV + THREADS - 1) / THREADS; ++q) {
        const int idx = threadIdx.x + q * THREADS;
        if (NV % THREADS == 0 || idx < NV) {
            int4 v = reinterpret_cast<const int4*>(src)[idx];
            v.x += 1;
            v.y += 1;
            v.z += 1;
            v.w += 1;
            reinterpret_cast<int4*>(dst)[idx] = v;
        }
    }
}

// The table route for a whole tile whose int32 values (the tile's in, halo included) lie in
// [lo, hi]: `nsteps` applications. The int32 tile takes half of the FP64 stage, so the other half
// holds the next application's in: while application t reads one, in + 1 goes to the other, and
// one barrier per application separates them; *fin (0 or SW * SH) is where the last application's
// in is left for the stores. Lane l owns columns l and l + 32 of its warp's rows; every application
// adds its S into their out words in o_s, a shared-memory tile of out words (row stride TW). With
// OUT_SMEM, o_s is the TMA kernel's out tile, which the stores then read in their own layout; with
// the other sources o_s is scratch, filled from the out array (out_g points at the tile's (0, 0),
// row stride n) before the first application and written back after the last, each thread its own
// points. Returns false, having done nothing, when the values span TBL_L or more (lo and hi are
// block-uniform). ONE: the launch applies the stencil once (the fixed-point share of one application).
template <int P, int R, int SW, int SH, int TW, int ROWS, int OUT_SRC, bool ONE>
__device__ __forceinline__ bool table_tile(int32_t* si, uint64_t* o_s, uint64_t* out_g, unsigned char* tbl, int lo,
                                           int hi, int nsteps, int64_t i0, int64_t j0, int64_t n, int64_t goff,
                                           int64_t row_end, bool has_out, int* fin)
{
    constexpr int ELEMS = SW * SH;
    static_assert(TW == 64, "two columns per lane, 32 apart");
    static_assert(ELEMS % 4 == 0, "the advance moves 16-byte vectors");
    if (hi - lo >= TBL_L) return false;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t* T64 = reinterpret_cast<uint64_t*>(tbl);
    uint4* T96 = reinterpret_cast<uint4*>(tbl + group_count<P, R>() * TBL_L * 8);
    int base = lo;
    build_tables<P, R>(T64, T96, base);
    if constexpr (OUT_SRC != OUT_SMEM) {
#pragma unroll
        for (int rr = 0; rr < ROWS; ++rr) {
            const int r = warp * ROWS + rr;
            const int64_t gi = i0 + r;
            if (!table_row_active(has_out, gi, gi + goff, row_end, n, R)) continue;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = lane + 32 * h;
                if (j0 + c >= R && j0 + c < n - R) o_s[r * TW + c] = out_g[r * n + c];
            }
        }
    }
    __syncthreads();  // the tables complete
    int cur = 0;
#pragma unroll 1
    for (int t = 0; t < nsteps; ++t) {
        if (t > 0 && hi + t >= base + TBL_L) {  // the values outgrew the table: rebuild it at the new minimum
            base = lo + t;
            build_tables<P, R>(T64, T96, base);
            __syncthreads();
        }
        const int32_t* s0 = si + cur + R * SW + ((SW - TW) / 2);  // the tile's (0, 0)
#pragma unroll 1
        for (int rr = 0; rr < ROWS; ++rr) {
            const int r = warp * ROWS + rr;
            const int64_t gi = i0 + r;
            if (!table_row_active(has_out, gi, gi + goff, row_end, n, R)) continue;  // warp-uniform
            double d[2];
            table_chain<P, R, SW, ONE>(s0 + r * SW + lane, T64, T96, base, d);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = lane + 32 * h;
                if (j0 + c >= R && j0 + c < n - R)
                    o_s[r * TW + c] = as_bits(__dadd_rn(as_dbl(o_s[r * TW + c]), d[h]));
            }
        }
        if (t + 1 < nsteps) {
            advance_i32_to<ELEMS>(si + cur, si + (ELEMS - cur));
            cur = ELEMS - cur;
            __syncthreads();  // the next application's in complete, this one's reads done
        }
    }
    *fin = cur;
    if constexpr (OUT_SRC != OUT_SMEM) {
#pragma unroll
        for (int rr = 0; rr < ROWS; ++rr) {
            const int r = warp * ROWS + rr;
            const int64_t gi = i0 + r;
            if (!table_row_active(has_out, gi, gi + goff, row_end, n, R)) continue;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = lane + 32 * h;
                if (j0 + c >= R && j0 + c < n - R) out_g[r * n + c] = o_s[r * TW + c];
            }
        }
    }
    __syncthreads();  // the out tile complete before the stores read it in their layout
    return true;
}

// ---------------------------------------------------------------------------------------------
// The kernel

// True when the tile at (i0, j0) holds interior points, i.e. has an out tile to load and update.
__device__ __forceinline__ bool tile_has_out(int64_t i0, int64_t j0, int64_t n, int R, int tw, int th)
{
    return (i0 + th > R) && (i0 < n - R) && (j0 + tw > R) && (j0 < n - R);
}


// Evaluate one tile whose `in` (with halo) is in shared memory: STEPS applications (`depth` when
// STEPS = 0), then in_next and out to HBM, with out read from OUT_SRC. vec_ok: rows are 16-byte
// aligned and n is a multiple of CPT, so a thread's CPT points move as one vector; otherwise they
// move one by one.
// The arrays hold rows of an n x n grid (row stride n); i0 is the tile's first row in the arrays and
// goff the grid row of the arrays' row 0 (0 for a whole grid; a row slab's first row otherwise).
// Rows from row_end on (in the arrays) are not stored; the interior test uses grid rows.
template <int P, int R, int DT, int STEPS, int OUT_SRC = OUT_SMEM, int TH_ = 32>
__device__ __forceinline__ void process_tile(unsigned char* stage, int* s_red, int64_t i0, int64_t j0, int64_t n,
                                             bool has_out, void* __restrict__ in_next_v, void* __restrict__ out_v,
                                             bool vec_ok, int depth, int64_t goff, int64_t row_end,
                                             unsigned char* tbl)
{
    const int nsteps = STEPS > 0 ? STEPS : depth;
    using G = Geo<DT, R, TH_>;
    using C = Cfg<DT, TH_>;
    using T = typename C::T;
    constexpr int CPT = C::CPT;
    constexpr int ROWS = G::ROWS;
    constexpr bool EXACT = DT == FP64 && pow2_weights(P, R);
    T* s_in = reinterpret_cast<T*>(stage);
    uint64_t* o_tile = reinterpret_cast<uint64_t*>(stage + G::OUT_OFF);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c0 = lane * CPT;
    const int64_t gj = j0 + c0;
    const bool col_ok = gj < n;  // at least the first of the thread's CPT columns is in the grid
    const bool cols_interior = gj >= R && gj + CPT <= n - R;
    // the out word of point (r, c0 + k), from the smem out tile or from HBM
    auto load_out = [&](int r, int k) -> uint64_t {
        if constexpr (OUT_SRC != OUT_SMEM) {
            return gj + k < n ? static_cast<const uint64_t*>(out_v)[(i0 + r) * n + gj + k] : 0ull;
        } else {
            return o_tile[r * C::TW + c0 + k];
        }
    };
    // the CPT out words of row r: from HBM as 16-byte vectors where the row's words start on a 16-byte
    // boundary and lie inside the grid (every other row when n is odd), else one by one
    auto load_out_row = [&](int r, uint64_t (&o)[CPT]) {
        if constexpr (OUT_SRC != OUT_SMEM) {
            const uint64_t* src = static_cast<const uint64_t*>(out_v) + (i0 + r) * n + gj;
            if (gj + CPT <= n && (reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
#pragma unroll
                for (int k = 0; k < CPT; k += 2) {
                    const ulonglong2 w = *reinterpret_cast<const ulonglong2*>(src + k);
                    o[k] = w.x;
                    o[k + 1] = w.y;
                }
                return;
            }
        }
#pragma unroll
        for (int k = 0; k < CPT; ++k) o[k] = load_out(r, k);
    };

    // ---- FP64 power-of-two stencils: certify the tile for an exact route ----
    // First the FP32 route: every value +0 or an integer of magnitude below 2^20 (checked with a few
    // integer ops and one FP32 round trip, no binary64 instruction). Otherwise the general integer
    // route (lowest-set-bit classification, int32/int64 arithmetic), otherwise strict binary64.
    int unit = fx::NOT_FIXED;
    bool narrow = false;
    bool fexact = false;
    if constexpr (EXACT) {
        constexpr int SHIFT = pow2_shift(P, R);
        constexpr long long L1 = pow2_coef_l1(P, R);
        constexpr int PER = (G::ELEMS + THREADS - 1) / THREADS;
        // FP32 route bound: L1 * (2^20 + steps) < 2^24 for L1 <= 15 and steps <= FP32_MAX_STEPS
        static_assert(L1 < 16 && STEPS <= FP32_MAX_STEPS, "FP32 route bound");
        const uint64_t* raw = reinterpret_cast<const uint64_t*>(s_in);
        float fv[PER];
        bool ok = true;
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int idx = threadIdx.x + q * THREADS;
            const uint64_t b = idx < G::ELEMS ? raw[idx] : 0ull;
            const uint32_t hi32 = static_cast<uint32_t>(b >> 32), lo32 = static_cast<uint32_t>(b);
            const uint32_t e = (hi32 >> 20) & 0x7FFu;
            const bool small = e >= 1023u && e < 1043u && (lo32 & 0x1FFFFFFFu) == 0u;
            const float f = __uint_as_float((hi32 & 0x80000000u) | (((hi32 & 0x7FFFFFFFu) - (896u << 20)) << 3) | (lo32 >> 29));
            const float fr = __fsub_rn(__fadd_rn(f, 12582912.0f), 12582912.0f);  // nearest integer, |f| < 2^22
            ok = ok && (b == 0ull || (small && fr == f));
            fv[q] = b == 0ull ? 0.0f : f;
        }
        if (STEPS == 0 && nsteps > FP32_MAX_STEPS) ok = false;
        ok = __syncthreads_and(ok) != 0;
        if (ok) {
            float* sf = reinterpret_cast<float*>(s_in);
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                const int idx = threadIdx.x + q * THREADS;
                if (idx < G::ELEMS) sf[idx] = fv[q];
            }
            fexact = true;
        } else {
            int lo = fx::ZERO_LO, hi = fx::ZERO_HI;
            for (int idx = threadIdx.x; idx < G::ELEMS; idx += THREADS) {
                int l, h;
                fx::classify(raw[idx], l, h);
                lo = min(lo, l);
                hi = max(hi, h);
            }
            lo = __reduce_min_sync(0xffffffffu, lo);
            hi = __reduce_max_sync(0xffffffffu, hi);
            if (lane == 0) {
                s_red[2 * warp] = lo;
                s_red[2 * warp + 1] = hi;
            }
            __syncthreads();
            lo = s_red[0];
            hi = s_red[1];
#pragma unroll
            for (int w = 1; w < WARPS; ++w) {
                lo = min(lo, s_red[2 * w]);
                hi = max(hi, s_red[2 * w + 1]);
            }
            unit = fx::certify(lo, hi, SHIFT, L1, nsteps);
            if (unit != fx::NOT_FIXED) {
                // int32 arithmetic suffices when every partial sum and every updated value stays below 2^31
                const int span = hi == fx::ZERO_HI ? 0 : hi + 1 - unit;
                narrow = span <= 30 && -unit <= 26 &&
                         ((1ll << span) + static_cast<long long>(nsteps) * (1ll << (-unit))) < (1ll << 31) / L1;
                __syncthreads();  // every thread has read its raw words
                int64_t* iv = reinterpret_cast<int64_t*>(s_in);
                for (int idx = threadIdx.x; idx < G::ELEMS; idx += THREADS) iv[idx] = fx::to_fixed(raw[idx], unit);
            }
        }
        __syncthreads();  // every converted word visible
    }
    // ---- FP64, other weights: whole-number tiles take their products off the binary64 pipe ----
    // Every value +0 or a whole number below 2^19 (so that up to 2^19 applications of in += 1 stay
    // below 2^20): the tile is held as int32 and fp64_points_whole evaluates it.
    bool iwhole = false;
    if constexpr (DT == FP64 && !EXACT) {
        constexpr int PER = (G::ELEMS + THREADS - 1) / THREADS;
        const uint64_t* raw = reinterpret_cast<const uint64_t*>(s_in);
        int32_t iv[PER];
        bool ok = nsteps <= (1 << 19);
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int idx = threadIdx.x + q * THREADS;
            const uint64_t b = idx < G::ELEMS ? raw[idx] : 0ull;
            const int e = static_cast<int>((b >> 52) & 0x7FF);
            const int sh = 1075 - e;  // fraction bits below the binary point, 34..52 in range
            const bool in_range = e >= 1023 && e <= 1041;
            const uint64_t m = (b & fx::MANT) | fx::HIDDEN;
            const bool whole = in_range && (m & ((1ull << (sh & 63)) - 1)) == 0;
            const int32_t a = in_range ? static_cast<int32_t>(m >> (sh & 63)) : 0;
            iv[q] = b == 0ull ? 0 : ((b >> 63) ? -a : a);
            ok = ok && (b == 0ull || whole);
        }
        if constexpr (table_route<P, R, DT>()) {
            // the tile's range for the table route, published with the certification's barrier
            int lo = 0x7FFFFFFF, hi = -0x7FFFFFFF;
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                if (threadIdx.x + q * THREADS < G::ELEMS) {
                    lo = min(lo, iv[q]);
                    hi = max(hi, iv[q]);
                }
            }
            lo = __reduce_min_sync(0xffffffffu, lo);
            hi = __reduce_max_sync(0xffffffffu, hi);
            if (lane == 0) {
                s_red[2 * warp] = lo;
                s_red[2 * warp + 1] = hi;
            }
        }
        iwhole = __syncthreads_and(ok) != 0;
        if (iwhole) {
            int32_t* si = reinterpret_cast<int32_t*>(s_in);
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                const int idx = threadIdx.x + q * THREADS;
                if (idx < G::ELEMS) si[idx] = iv[q];
            }
        }
        __syncthreads();
    }

    // ---- FP64, other weights: the table route (table_tile), when the kernel has a table area and
    // the tile's range fits it ----
    bool tbl_done = false;
    int iw_fin = 0;  // where the int32 tile of the last application's in lies (int32 elements)
    if constexpr (table_route<P, R, DT>()) {
        if (iwhole && tbl) {
            int lo = s_red[0], hi = s_red[1];
#pragma unroll
            for (int w = 1; w < WARPS; ++w) {
                lo = min(lo, s_red[2 * w]);
                hi = max(hi, s_red[2 * w + 1]);
            }
            // kernels that keep out in HBM give the route an out area right after the tables
            uint64_t* o_s = OUT_SRC == OUT_SMEM ? o_tile : reinterpret_cast<uint64_t*>(tbl + table_bytes<P, R, DT>());
            tbl_done = table_tile<P, R, G::SW, G::SH, C::TW, ROWS, OUT_SRC, STEPS == 1>(
                reinterpret_cast<int32_t*>(s_in), o_s, static_cast<uint64_t*>(out_v) + i0 * n + j0, tbl, lo, hi,
                nsteps, i0, j0, n, goff, row_end, has_out, &iw_fin);
        }
    }

    // The table route with out in HBM has stored out itself; the stores then write in_next only
    const bool out_via_rows = !(tbl_done && OUT_SRC != OUT_SMEM);

    // Set by the multi-application FP32 route when the tile's out words are held as integers
    bool oint = false;
    // Offset in floats of the FP32 tile holding the last application's in (double-buffered route)
    int fin_off = 0;

    // S of CPT points of row r (tile coordinates) added into the out words o[] (in place)
    auto apply_row = [&](int r, uint64_t* o) {
        const int soff = (r + R) * G::SW + G::RA + c0;  // in(r, c0) in the tile
        if constexpr (DT == FP64) {
            bool done = false;
            if constexpr (EXACT) {
                constexpr int SHIFT = pow2_shift(P, R);
                const int64_t* v = reinterpret_cast<const int64_t*>(s_in) + soff;
                if (fexact) {
                    float S[CPT];
                    fexact_points<P, R, CPT, G::RA>(reinterpret_cast<const float*>(s_in) + soff, G::SW, S);
                    if (oint) {
#pragma unroll
                        for (int k = 0; k < CPT; ++k) {
                            if constexpr (STEPS == 0)
                                o[k] += static_cast<uint64_t>(static_cast<int64_t>(__float2int_rn(S[k])));
                            else
                                o[k] = static_cast<uint32_t>(static_cast<uint32_t>(o[k]) + static_cast<uint32_t>(__float2int_rn(S[k])));
                        }
                    } else {
#pragma unroll
                        for (int k = 0; k < CPT; ++k) o[k] = as_bits(__dadd_rn(as_dbl(o[k]), as_dbl(f2d(S[k], -SHIFT))));
                    }
                    done = true;
                } else if (unit != fx::NOT_FIXED) {
                    if (narrow) {
                        int32_t S[CPT];
                        fx_points<P, R, CPT, G::RA>(v, G::SW, S);
#pragma unroll
                        for (int k = 0; k < CPT; ++k)
                            o[k] = as_bits(__dadd_rn(as_dbl(o[k]), as_dbl(from_fixed32(S[k], unit - SHIFT))));
                    } else {
                        int64_t S[CPT];
                        fx_points<P, R, CPT, G::RA>(v, G::SW, S);
#pragma unroll
                        for (int k = 0; k < CPT; ++k)
                            o[k] = as_bits(__dadd_rn(as_dbl(o[k]), as_dbl(fx::from_fixed(S[k], unit - SHIFT))));
                    }
                    done = true;
                }
            }
            if constexpr (!EXACT) {
                if (iwhole) {
                    double S[CPT];
                    fp64_points_whole<P, R, G::SW, CPT>(reinterpret_cast<const int32_t*>(s_in) + soff, S);
#pragma unroll
                    for (int k = 0; k < CPT; ++k) o[k] = as_bits(__dadd_rn(as_dbl(o[k]), S[k]));
                    done = true;
                }
            }
            if (!done) {
                const double* sp = reinterpret_cast<const double*>(s_in) + soff;
#pragma unroll
                for (int k = 0; k < CPT; ++k) o[k] = as_bits(__dadd_rn(as_dbl(o[k]), fp64_point<P, R>(sp + k, G::SW)));
            }
        } else {
            const float* sp = reinterpret_cast<const float*>(s_in) + soff;
            float sh[CPT], sl[CPT];
            fp32c_points<P, R, CPT, G::RA>(sp, G::SW, sh, sl);
#pragma unroll
            for (int k = 0; k < CPT; ++k) {
                float oh = __uint_as_float(static_cast<uint32_t>(o[k]));
                float ol = __uint_as_float(static_cast<uint32_t>(o[k] >> 32));
                if constexpr (STEPS == 1)
                    df_add(oh, ol, sh[k], sl[k]);
                else  // out stays in registers: renormalised once, before it is stored
                    df_add_lazy(oh, ol, sh[k], sl[k]);
                o[k] = static_cast<uint64_t>(__float_as_uint(oh)) | (static_cast<uint64_t>(__float_as_uint(ol)) << 32);
            }
        }
    };

    // in_next (in + 1 after the last application) and out of row r to HBM
    auto store_row = [&](int r, const uint64_t* o, bool row_out) {
        const int64_t gi = i0 + r;
        const int soff = (r + R) * G::SW + G::RA + c0;
        T nxt[CPT];
        bool done = false;
        if constexpr (EXACT) {
            if (fexact) {
                const float* v = reinterpret_cast<const float*>(s_in) + fin_off + soff;
#pragma unroll
                for (int k = 0; k < CPT; ++k) nxt[k] = as_dbl(f2d(__fadd_rn(v[k], 1.0f), 0));
                done = true;
            } else if (unit != fx::NOT_FIXED) {
                const int64_t* v = reinterpret_cast<const int64_t*>(s_in) + soff;
                const int64_t one = 1ll << (-unit);
                if (narrow) {
#pragma unroll
                    for (int k = 0; k < CPT; ++k) nxt[k] = as_dbl(from_fixed32(static_cast<int32_t>(v[k] + one), unit));
                } else {
#pragma unroll
                    for (int k = 0; k < CPT; ++k) nxt[k] = as_dbl(fx::from_fixed(v[k] + one, unit));
                }
                done = true;
            }
        }
        if constexpr (DT == FP64 && !EXACT) {
            if (iwhole) {
                const int32_t* v = reinterpret_cast<const int32_t*>(s_in) + iw_fin + soff;
#pragma unroll
                for (int k = 0; k < CPT; ++k) nxt[k] = as_dbl(from_fixed32(v[k] + 1, 0));
                done = true;
            }
        }
        if (!done) {
#pragma unroll
            for (int k = 0; k < CPT; ++k) {
                if constexpr (DT == FP64)
                    nxt[k] = inc_exact(s_in[soff + k]);
                else
                    nxt[k] = __fadd_rn(s_in[soff + k], 1.0f);
            }
        }
        T* nx = static_cast<T*>(in_next_v) + gi * n + gj;
        // 16-byte stores wherever the row's words start on a 16-byte boundary inside the grid (every
        // row for the TMA tiles; every other row for an odd n)
        if (vec_ok || (gj + CPT <= n && (reinterpret_cast<uintptr_t>(nx) & 15u) == 0)) {
            st_vec(nx, nxt);
        } else {
#pragma unroll
            for (int k = 0; k < CPT; ++k)
                if (gj + k < n) nx[k] = nxt[k];
        }
        if (row_out) {
            uint64_t* out = static_cast<uint64_t*>(out_v) + gi * n + gj;
            if (cols_interior && (vec_ok || (reinterpret_cast<uintptr_t>(out) & 15u) == 0)) {
#pragma unroll
                for (int k = 0; k < CPT; k += 2) *reinterpret_cast<ulonglong2*>(out + k) = make_ulonglong2(o[k], o[k + 1]);
            } else {
#pragma unroll
                for (int k = 0; k < CPT; ++k)
                    if (gj + k >= R && gj + k < n - R) out[k] = o[k];
            }
        }
    };

    if constexpr (STEPS == 1) {
        // one pass: each row's new out and in_next leave as soon as they are computed. OUT_HBM_AHEAD:
        // every row's out words are requested first, so that their latencies overlap instead of
        // stalling each row in turn.
        constexpr bool PRELOAD = OUT_SRC == OUT_HBM_AHEAD && EXACT;
        uint64_t o_pre[PRELOAD ? ROWS : 1][CPT];
        if constexpr (PRELOAD) {
#pragma unroll
            for (int rr = 0; rr < ROWS; ++rr) {
                const int r = warp * ROWS + rr;
                const int64_t gi = i0 + r, gg = gi + goff;
                const bool row_out = col_ok && gi < row_end && has_out && gg >= R && gg < n - R;
                if (row_out) {
                    load_out_row(r, o_pre[rr]);
                } else {
#pragma unroll
                    for (int k = 0; k < CPT; ++k) o_pre[rr][k] = 0ull;
                }
            }
        }
#pragma unroll
        for (int rr = 0; rr < ROWS; ++rr) {
            const int r = warp * ROWS + rr;
            const int64_t gi = i0 + r, gg = gi + goff;
            if (!col_ok || gi >= row_end) continue;
            const bool row_out = out_via_rows && has_out && gg >= R && gg < n - R;
            uint64_t o[CPT];
            if (row_out) {
                if constexpr (PRELOAD) {
#pragma unroll
                    for (int k = 0; k < CPT; ++k) o[k] = o_pre[rr][k];
                } else {
                    load_out_row(r, o);
                }
                if (!tbl_done) apply_row(r, o);
            }
            store_row(r, o, row_out);
        }
    } else {
        // out of the thread's points stays in registers across the applications
        static_assert(G::ELEMS % 4 == 0, "the in-place advance moves 16-byte vectors");
        uint64_t o[ROWS][CPT];
        bool ract[ROWS];  // the row holds interior points
#pragma unroll
        for (int rr = 0; rr < ROWS; ++rr) {
            const int r = warp * ROWS + rr;
            const int64_t gi = i0 + r, gg = gi + goff;
            ract[rr] = out_via_rows && col_ok && gi < row_end && has_out && gg >= R && gg < n - R;
            if (ract[rr]) {
                load_out_row(r, o[rr]);
            } else {
#pragma unroll
                for (int k = 0; k < CPT; ++k) o[rr][k] = 0ull;
            }
        }
        if constexpr (EXACT) {
            // FP32 route: when every out word the tile stores is an integer V of 2^-SHIFT units with
            // |V| < 2^21, out is held as V. Every S is an integer below 2^24 units, so each binary64
            // add of the reference chain (out + S) is exact (the running V stays below 2^28 for 8
            // applications, int32, and below 2^41 for FP32_MAX_STEPS, int64) and its conversion at
            // the end gives the same bits; a zero comes out +0 both ways (S is never -0). The
            // applications then add integers instead of issuing binary64 adds.
            if (fexact) {
                constexpr int SHIFT = pow2_shift(P, R);
                int32_t V[ROWS][CPT];
                bool ok = true;
#pragma unroll
                for (int rr = 0; rr < ROWS; ++rr) {
#pragma unroll
                    for (int k = 0; k < CPT; ++k) {
                        const bool fits = out_units(o[rr][k], SHIFT, V[rr][k]);
                        const bool stored = ract[rr] && gj + k >= R && gj + k < n - R;
                        ok = ok && (!stored || fits);
                    }
                }
                oint = __syncthreads_and(ok) != 0;
                if (oint) {
#pragma unroll
                    for (int rr = 0; rr < ROWS; ++rr)
#pragma unroll
                        for (int k = 0; k < CPT; ++k) {
                            if constexpr (STEPS == 0)
                                o[rr][k] = static_cast<uint64_t>(static_cast<int64_t>(V[rr][k]));
                            else  // V in the low word, high word zero
                                o[rr][k] = static_cast<uint32_t>(V[rr][k]);
                        }
                }
            }
        }
        bool fast = false;  // the FP32 route with integer-held out (block-uniform)
        if constexpr (EXACT) fast = fexact && oint;
        if (fast) {
            // The same applications in their tightest form: the route is fixed for the launch, and
            // a thread's S for all its rows comes from one pass over its column strip. The FP32
            // tile takes half of the binary64 stage, so the other half holds the next
            // application's in: while application t reads one, in + 1 is written to the other (each
            // thread its own points, from the values it has just read, and the threads together
            // the halo), and one barrier per application separates them.
            if constexpr (EXACT) {
                float* const buf = reinterpret_cast<float*>(s_in);
                const int own = (warp * ROWS + R) * G::SW + G::RA + c0;
#pragma unroll 1
                for (int t = 0; t < nsteps; ++t) {
                    const int cur = (t & 1) * G::ELEMS;
                    float S[ROWS][CPT], v[ROWS][CPT];
                    fexact_rows<P, R, CPT, ROWS, G::RA>(buf + cur + own, G::SW, S, v);
                    if (t + 1 < nsteps) {
                        float* nx = buf + (G::ELEMS - cur);
#pragma unroll
                        for (int rr = 0; rr < ROWS; ++rr) {
                            static_assert(CPT == 2, "own points move as one 8-byte pair");
                            *reinterpret_cast<float2*>(nx + own + rr * G::SW) =
                                make_float2(__fadd_rn(v[rr][0], 1.0f), __fadd_rn(v[rr][1], 1.0f));
                        }
                        advance_halo_f32<G::SW, G::SH, R, G::RA>(buf + cur, nx);
                        __syncthreads();
                    }
#pragma unroll
                    for (int rr = 0; rr < ROWS; ++rr)
#pragma unroll
                        for (int k = 0; k < CPT; ++k) {
                            if constexpr (STEPS == 0)
                                o[rr][k] += static_cast<uint64_t>(static_cast<int64_t>(__float2int_rn(S[rr][k])));
                            else
                                o[rr][k] = static_cast<uint32_t>(static_cast<uint32_t>(o[rr][k]) +
                                                                 static_cast<uint32_t>(__float2int_rn(S[rr][k])));
                        }
                }
                fin_off = ((nsteps - 1) & 1) * G::ELEMS;
            }
        } else if (!tbl_done) {
#pragma unroll 1
        for (int t = 0; t < nsteps; ++t) {
            if (t > 0) {  // advance the whole tile, halo included: in_{k+1} = in_k + 1
                __syncthreads();
                if constexpr (DT == FP64) {
                    bool adv = false;
                    if constexpr (EXACT) {
                        if (fexact) {
                            advance_f32<G::ELEMS>(reinterpret_cast<float*>(s_in));
                            adv = true;
                        } else if (unit != fx::NOT_FIXED) {
                            advance_i64<G::ELEMS>(reinterpret_cast<int64_t*>(s_in), 1ll << (-unit));
                            adv = true;
                        }
                    }
                    if constexpr (!EXACT) {
                        if (iwhole) {
                            advance_i32<G::ELEMS>(reinterpret_cast<int32_t*>(s_in));
                            adv = true;
                        }
                    }
                    if (!adv) advance_f64<G::ELEMS>(s_in);
                } else {
                    advance_f32<G::ELEMS>(s_in);
                }
                __syncthreads();
            }
#pragma unroll
            for (int rr = 0; rr < ROWS; ++rr)
                if (ract[rr]) apply_row(warp * ROWS + rr, o[rr]);
        }
        }
        if constexpr (DT == FP32C) {  // the pairs accumulated without renormalising
#pragma unroll
            for (int rr = 0; rr < ROWS; ++rr)
#pragma unroll
                for (int k = 0; k < CPT; ++k) {
                    float oh, ol;
                    fast_two_sum(__uint_as_float(static_cast<uint32_t>(o[rr][k])),
                                 __uint_as_float(static_cast<uint32_t>(o[rr][k] >> 32)), oh, ol);
                    o[rr][k] = static_cast<uint64_t>(__float_as_uint(oh)) |
                               (static_cast<uint64_t>(__float_as_uint(ol)) << 32);
                }
        }
        if (oint) {
#pragma unroll
            for (int rr = 0; rr < ROWS; ++rr)
#pragma unroll
                for (int k = 0; k < CPT; ++k) {
                    if constexpr (STEPS == 0)
                        o[rr][k] = fx::from_fixed(static_cast<int64_t>(o[rr][k]), -pow2_shift(P, R));
                    else
                        o[rr][k] = from_fixed32(static_cast<int32_t>(static_cast<uint32_t>(o[rr][k])), -pow2_shift(P, R));
                }
        }
#pragma unroll
        for (int rr = 0; rr < ROWS; ++rr) {
            const int r = warp * ROWS + rr;
            const int64_t gi = i0 + r, gg = gi + goff;
            if (!col_ok || gi >= row_end) continue;
            store_row(r, o[rr], out_via_rows && has_out && gg >= R && gg < n - R);
        }
    }
}

#ifndef PRK_STRICT_BLOCKS_1
#define PRK_STRICT_BLOCKS_1 3
#endif
#ifndef PRK_STRICT_BLOCKS_N
#define PRK_STRICT_BLOCKS_N 3
#endif

// Register budget: the single-application kernels keep as many tiles resident as shared memory
// allows, so that every SM has enough loads in flight; the multi-application kernels hold `out` in
// registers and run at most four tiles per SM. The strict FP64 form is bound by the binary64 pipe
// and gets the registers its unrolled tap sequence wants.
template <int P, int R, int DT, int STEPS, int TH_>
constexpr int min_blocks()
{
    // the table route: three tiles per SM (80 registers), so that 24 warps hide the fixed-point
    // chains' latencies (at four, 64 registers, the longer chains spill); tiles whose shared memory
    // (tile and tables) admits at most two per SM get the registers of two (the 64-row tiles of grid
    // R=3..5: at three, grid R=5 spilled 3 KB)
    if (DT == FP64 && !pow2_weights(P, R)) {
        if (SMEM_PER_SM / (tile_smem<P, R, DT, TH_>() + 1024) < 3) return 2;
        return STEPS == 1 ? PRK_STRICT_BLOCKS_1 : PRK_STRICT_BLOCKS_N;
    }
    if (DT == FP32C && P == GRID && R >= 3) return 2;  // bound by FP32 issue: registers over residency
    const int b = Geo<DT, R, TH_>::CTAS;
    if (STEPS == 1) return b;
    const int cap = DT == FP64 ? 4 : 3;  // FP64 power-of-two: the FP32 route is shared-memory bound
    return b < cap ? b : cap;
}

// One CTA per tile: blockIdx = (tile column, tile row). The elected thread issues the tile's two TMA
// loads; every thread waits on the mbarrier with a bounded spin, and on a timeout the CTA flags
// `status`, waits (again bounded) for the copies to land and returns. The arrays hold rows of the
// n x n grid from grid row goff (the tensor maps cover exactly the rows they hold, so the hardware
// zero-fills anything beyond); rows from row_end on are read as halo but not stored.
template <int P, int R, int DT, int STEPS, int TH_>
__global__ void __launch_bounds__(THREADS, min_blocks<P, R, DT, STEPS, TH_>())
    k_stencil_tile(const __grid_constant__ CUtensorMap tm_in, const __grid_constant__ CUtensorMap tm_out,
                   const int64_t n, void* __restrict__ in_next_v, void* __restrict__ out_v, unsigned* __restrict__ status,
                   const int depth, const int64_t row0, const int64_t goff, const int64_t row_end)
{
    using G = Geo<DT, R, TH_>;
    using C = Cfg<DT, TH_>;
    extern __shared__ __align__(128) unsigned char smem[];
    int* s_red = reinterpret_cast<int*>(smem + G::RED_OFF);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + G::BAR_OFF);
    const int64_t i0 = row0 + static_cast<int64_t>(blockIdx.y) * C::TH;
    const int64_t j0 = static_cast<int64_t>(blockIdx.x) * C::TW;
    const bool has_out = tile_has_out(i0 + goff, j0, n, R, C::TW, C::TH);

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        mbar_arrive_expect_tx(bar, G::IN_BYTES + (has_out ? G::OUT_BYTES : 0));
        tma_load_2d(smem, &tm_in, static_cast<int32_t>(j0 - G::RA), static_cast<int32_t>(i0 - R), bar);
        if (has_out) tma_load_2d(smem + G::OUT_OFF, &tm_out, static_cast<int32_t>(j0), static_cast<int32_t>(i0), bar);
    }
    __syncthreads();
    // One decision for the whole CTA: process_tile's barriers need every thread, so the tile is
    // evaluated only when every thread saw the loads land.
    if (!__syncthreads_and(mbar_wait_bounded(bar, 0))) {
        if (threadIdx.x == 0) atomicOr(status, 1u);
        mbar_wait_bounded(bar, 0);  // let the copies land before the CTA's shared memory is released
        return;
    }
    process_tile<P, R, DT, STEPS, OUT_SMEM, TH_>(smem, s_red, i0, j0, n, has_out, in_next_v, out_v, true, depth, goff,
                                                 row_end,
                                                 table_route<P, R, DT>() ? smem + table_offset<DT, R, TH_>() : nullptr);
}

template <int P, int R, int DT, int STEPS, int TH_>
cudaError_t launch(const Launch& L)
{
    using C = Cfg<DT, TH_>;
    constexpr int SMEM = tile_smem<P, R, DT, TH_>();
    static_assert(SMEM <= SMEM_PER_CTA_MAX, "the tile and its tables must fit in shared memory");
    if (cudaError_t e = cudaFuncSetAttribute(k_stencil_tile<P, R, DT, STEPS, TH_>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM))
        return e;
    const int64_t nr = L.nr > 0 ? L.nr : L.n;
    if (L.row0 < 0 || L.row0 >= nr || L.rows < 0 || (STEPS == 0 && L.depth < 1) || L.goff < 0 || L.goff + nr > L.n)
        return cudaErrorInvalidValue;
    const int64_t rows = L.rows > 0 && L.rows < nr - L.row0 ? L.rows : nr - L.row0;
    const int64_t tx = (L.n + C::TW - 1) / C::TW, ty = (rows + C::TH - 1) / C::TH;
    if (ty > 65535) return cudaErrorInvalidValue;
    const dim3 grid(static_cast<unsigned>(tx), static_cast<unsigned>(ty));
    k_stencil_tile<P, R, DT, STEPS, TH_><<<grid, THREADS, SMEM, L.stream>>>(L.tm_in, L.tm_out, L.n, L.in_next, L.out,
                                                                             L.status, L.depth, L.row0, L.goff,
                                                                             L.row0 + rows);
    return cudaGetLastError();
}

// Supported temporal depths; a run of any length is split into launches of these, or runs in one
// launch of the run-time-depth kernel (steps = 0, TH = 32 only).
constexpr int MAX_STEPS = 8;

template <int P, int DT, int TH_>
cudaError_t launch_pattern(int R, int steps, const Launch& L)
{
#define PRK_TILE_CASE(RR)                                        \
    case RR:                                                     \
        switch (steps) {                                         \
        case 1: return launch<P, RR, DT, 1, TH_>(L);             \
        case 2: return launch<P, RR, DT, 2, TH_>(L);             \
        case 4: return launch<P, RR, DT, 4, TH_>(L);             \
        case 8: return launch<P, RR, DT, 8, TH_>(L);             \
        case 0:                                                  \
            if constexpr (TH_ == TH_DEFAULT)                     \
                return launch<P, RR, DT, 0, TH_>(L);             \
            else                                                 \
                return cudaErrorInvalidValue;                    \
        default: return cudaErrorInvalidValue;                   \
        }
    switch (R) {
        PRK_TILE_CASE(1)
        PRK_TILE_CASE(2)
        PRK_TILE_CASE(3)
        PRK_TILE_CASE(4)
        PRK_TILE_CASE(5)
    }
#undef PRK_TILE_CASE
    return cudaErrorInvalidValue;
}

// Tile geometry for the host: box sizes of the two tensor maps for tile height th.
inline void boxes(int dtype, int R, int th, int* in_x, int* in_y, int* out_x, int* out_y)
{
    const int vec = dtype == FP64 ? 2 : 4;
    const int ra = ((R + vec - 1) / vec) * vec;
    const int tw = dtype == FP64 ? Cfg<FP64>::TW : Cfg<FP32C>::TW;
    *in_x = tw + 2 * ra;
    *in_y = th + 2 * R;
    *out_x = tw;
    *out_y = th;
}

// Per-translation-unit entry points (tile_*.cu), one per storage form, pattern and tile height.
cudaError_t launch_fp64_star(int R, int steps, const Launch& L);
cudaError_t launch_fp64_grid(int R, int steps, const Launch& L);
cudaError_t launch_fp32c_star(int R, int steps, const Launch& L);
cudaError_t launch_fp32c_grid(int R, int steps, const Launch& L);
cudaError_t launch_fp64_star_tall(int R, int steps, const Launch& L);
cudaError_t launch_fp64_grid_tall(int R, int steps, const Launch& L);
cudaError_t launch_fp32c_star_tall(int R, int steps, const Launch& L);
cudaError_t launch_fp32c_grid_tall(int R, int steps, const Launch& L);

}  // namespace tile
}  // namespace prk
