// Shared definitions for the GB300 stencil kernels: the PRK weight matrix, tap order and the small
// arithmetic helpers every form uses.
//
// Weights and tap order follow Cxx11/generate-cxx-stencil.py: instance() (:209-232) builds
// W[col+R][row+R]; bodygen() (:8-39) emits the nonzero taps with the column offset as the outer
// loop and the row offset as the inner loop, and the sum as ((t1 + t2) + ...) + tm added to out.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace prk {

enum Pattern : int { STAR = 0, GRID = 1 };
enum Dtype : int { FP64 = 0, FP32C = 1 };

constexpr int RMAX = 5;

// W[R+dc][R+dr] of generate-cxx-stencil.py:211-230. Star: +-1/(2kR) on the centre row and column.
// Grid: ring m = max(|dc|,|dr|) carries +-1/(4m(2m-1)R) on its sides and +-1/(4mR) on the main
// diagonal; anti-diagonal corners and the centre are zero. The sign is the sign of the offset that
// reaches the ring. Division by an integer is correctly rounded, as in the generator's Python.
__host__ __device__ constexpr double weight(int pattern, int R, int dc, int dr)
{
    if (pattern == STAR) {
        if (dc == 0 && dr != 0) return dr > 0 ? 1.0 / double(2 * dr * R) : -(1.0 / double(-2 * dr * R));
        if (dr == 0 && dc != 0) return dc > 0 ? 1.0 / double(2 * dc * R) : -(1.0 / double(-2 * dc * R));
        return 0.0;
    }
    const int adc = dc > 0 ? dc : -dc, adr = dr > 0 ? dr : -dr;
    const int m = adc > adr ? adc : adr;
    if (m == 0) return 0.0;
    if (adc == m && adr == m) {
        if (dc != dr) return 0.0;
        return dc > 0 ? 1.0 / double(4 * m * R) : -(1.0 / double(4 * m * R));
    }
    const double w = 1.0 / double(4 * m * (2 * m - 1) * R);
    if (adr == m) return dr > 0 ? w : -w;
    return dc > 0 ? w : -w;
}

// Integer denominator of |W| (0 for a zero tap). Every PRK weight is +-1/den.
__host__ __device__ constexpr int weight_den(int pattern, int R, int dc, int dr)
{
    if (pattern == STAR) {
        if (dc == 0 && dr != 0) return 2 * (dr > 0 ? dr : -dr) * R;
        if (dr == 0 && dc != 0) return 2 * (dc > 0 ? dc : -dc) * R;
        return 0;
    }
    const int adc = dc > 0 ? dc : -dc, adr = dr > 0 ? dr : -dr;
    const int m = adc > adr ? adc : adr;
    if (m == 0) return 0;
    if (adc == m && adr == m) return dc == dr ? 4 * m * R : 0;
    return 4 * m * (2 * m - 1) * R;
}

__host__ __device__ constexpr int weight_sign(int pattern, int R, int dc, int dr)
{
    const double w = weight(pattern, R, dc, dr);
    return w > 0.0 ? 1 : (w < 0.0 ? -1 : 0);
}

// PRK's stencil_size (stencil-openmp.cc:253): 4R+1 for star, (2R+1)^2 for grid.
__host__ __device__ constexpr int stencil_size(int pattern, int R)
{
    return pattern == STAR ? 4 * R + 1 : (2 * R + 1) * (2 * R + 1);
}

// Number of nonzero taps: star 4R, grid 4R^2 + 2R.
__host__ __device__ constexpr int tap_count(int pattern, int R)
{
    return pattern == STAR ? 4 * R : 4 * R * R + 2 * R;
}

// True when every |W| is a power of two (star R=1,2 and grid R=1): then w*x is exact in binary64.
__host__ __device__ constexpr bool pow2_weights(int pattern, int R)
{
    for (int dc = -R; dc <= R; ++dc)
        for (int dr = -R; dr <= R; ++dr) {
            const int d = weight_den(pattern, R, dc, dr);
            if (d != 0 && (d & (d - 1)) != 0) return false;
        }
    return true;
}

// log2 of the largest denominator when pow2_weights() holds: w * 2^shift is an integer for all taps.
__host__ __device__ constexpr int pow2_shift(int pattern, int R)
{
    int s = 0;
    for (int dc = -R; dc <= R; ++dc)
        for (int dr = -R; dr <= R; ++dr) {
            int d = weight_den(pattern, R, dc, dr), k = 0;
            while (d > 1) {
                d >>= 1;
                ++k;
            }
            if (k > s) s = k;
        }
    return s;
}

// Sum of |w * 2^pow2_shift| over the taps, an integer when pow2_weights() holds.
__host__ __device__ constexpr long long pow2_coef_l1(int pattern, int R)
{
    const int s = pow2_shift(pattern, R);
    long long t = 0;
    for (int dc = -R; dc <= R; ++dc)
        for (int dr = -R; dr <= R; ++dr) {
            const int d = weight_den(pattern, R, dc, dr);
            if (d != 0) t += (1LL << s) / d;
        }
    return t;
}

// Round a double to the nearest float and the float remainder: w = hi + lo to ~2^-48.
__host__ __device__ constexpr float split_hi(double w) { return static_cast<float>(w); }
__host__ __device__ constexpr float split_lo(double w) { return static_cast<float>(w - static_cast<double>(static_cast<float>(w))); }

}  // namespace prk
