/*
 * CPU restatement of the PRK 2D stencil hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle that the GPU path is checked against, and the
 * CPU baseline that the benchmark times beside it. The shipped library never links, loads or calls
 * it.  It is compiled twice (see oracle/Makefile):
 *
 *   liboracle.so  -O2 -ffp-contract=off, no fast-math: every product and sum is rounded once, in
 *                 the generator's tap order. This is the parity oracle.
 *   libprkcpu.so  -O3 -ffast-math -fopenmp: the reference's own compiler flags
 *                 (common/make.defs.gcc:14,20,37). This is the timed CPU baseline ("port").
 *
 * What it restates (paths are within the ParRes/Kernels project):
 *   - Cxx11/generate-cxx-stencil.py:209-232  weight matrix W[col+R][row+R] for star and grid;
 *   - Cxx11/generate-cxx-stencil.py:8-39     tap order: outer loop over the column offset -R..R,
 *                                            inner loop over the row offset -R..R, zeros skipped,
 *                                            out[i*n+j] += ((t1 + t2) + ...) + tm;
 *   - Cxx11/stencil_openmp.hpp:1-16          tiled loop nest over the interior R..n-R-1;
 *   - Cxx11/stencil-openmp.cc:182-223        init in=i+j, out=0; iterations+1 applications, each
 *                                            followed by in += 1.0 over the whole n x n; the timer
 *                                            starts at iteration 1;
 *   - Cxx11/stencil-openmp.cc:230-258        L1 norm over the interior / (n-2R)^2, check against
 *                                            2*(iterations+1) with epsilon 1e-8, flop count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PRK_STAR 0
#define PRK_GRID 1
#define PRK_RMAX 5

/* Weight of the tap at column offset dc and row offset dr, i.e. the generator's W[R+dc][R+dr]
 * (generate-cxx-stencil.py:211-230).  Star: +-1/(2kR) on the centre row and column.  Grid: ring
 * m = max(|dc|,|dr|) carries +-1/(4m(2m-1)R) on its four sides (the corner-free part) and
 * +-1/(4mR) on the main diagonal; the anti-diagonal corners and the centre are zero.  The sign is
 * the sign of the offset that reaches the ring. */
static inline __attribute__((always_inline)) double tap_weight(int pattern, int R, int dc, int dr)
{
    if (pattern == PRK_STAR) {
        if (dc == 0 && dr != 0) {
            int k = dr > 0 ? dr : -dr;
            double w = 1.0 / (double)(2 * k * R);
            return dr > 0 ? w : -w;
        }
        if (dr == 0 && dc != 0) {
            int k = dc > 0 ? dc : -dc;
            double w = 1.0 / (double)(2 * k * R);
            return dc > 0 ? w : -w;
        }
        return 0.0;
    }
    int adc = dc > 0 ? dc : -dc, adr = dr > 0 ? dr : -dr;
    int m = adc > adr ? adc : adr;
    if (m == 0) return 0.0;
    if (adc == m && adr == m) {
        if (dc != dr) return 0.0; /* anti-diagonal corner */
        double w = 1.0 / (double)(4 * m * R);
        return dc > 0 ? w : -w;
    }
    double w = 1.0 / (double)(4 * m * (2 * m - 1) * R);
    if (adr == m) return dr > 0 ? w : -w; /* row offset reaches the ring */
    return dc > 0 ? w : -w;               /* column offset reaches the ring */
}

double prk_oracle_weight(int pattern, int R, int dc, int dr) { return tap_weight(pattern, R, dc, dr); }

/* Taps in the generator's emission order. Returns the tap count (star 4R, grid 4R^2+2R). */
int prk_oracle_taps(int pattern, int R, int* dc_out, int* dr_out, double* w_out)
{
    int k = 0;
    for (int dc = -R; dc <= R; ++dc)
        for (int dr = -R; dr <= R; ++dr) {
            double w = tap_weight(pattern, R, dc, dr);
            if (w != 0.0) {
                if (dc_out) dc_out[k] = dc;
                if (dr_out) dr_out[k] = dr;
                if (w_out) w_out[k] = w;
                ++k;
            }
        }
    return k;
}

/* One stencil application over the interior, tiled by t, as an orphaned `omp for` over tiles
 * (stencil_openmp.hpp:2-15). With pattern and R compile-time constants, the unrolled tap loops
 * fold into the same straight-line expression the generator emits. */
#define DEFINE_APPLY_T(P, PNAME, RR, IDX, SUFFIX)                                                          \
    static void apply_##PNAME##RR##SUFFIX(const int64_t n64, const int64_t t64, const double* restrict in,  \
                                          double* restrict out)                                            \
    {                                                                                                     \
        const int R = RR;                                                                                 \
        const IDX n = (IDX)n64, t = (IDX)t64;                                                             \
        _Pragma("omp for collapse(2) schedule(static)")                                                   \
        for (IDX it = R; it < n - R; it += t) {                                                           \
            for (IDX jt = R; jt < n - R; jt += t) {                                                       \
                const IDX iend = (it + t < n - R) ? it + t : n - R;                                       \
                const IDX jend = (jt + t < n - R) ? jt + t : n - R;                                       \
                for (IDX i = it; i < iend; ++i) {                                                         \
                    _Pragma("omp simd")                                                                   \
                    for (IDX j = jt; j < jend; ++j) {                                                     \
                        double s = 0.0;                                                                   \
                        int first = 1;                                                                    \
                        _Pragma("GCC unroll 16")                                                          \
                        for (int dc = -R; dc <= R; ++dc) {                                                \
                            _Pragma("GCC unroll 16")                                                      \
                            for (int dr = -R; dr <= R; ++dr) {                                            \
                                const double w = tap_weight(P, R, dc, dr);                                \
                                if (w != 0.0) {                                                           \
                                    const double p = in[(i + dr) * n + (j + dc)] * w;                     \
                                    if (first) {                                                          \
                                        s = p;                                                            \
                                        first = 0;                                                        \
                                    } else {                                                              \
                                        s = s + p;                                                        \
                                    }                                                                     \
                                }                                                                         \
                            }                                                                             \
                        }                                                                                 \
                        out[i * n + j] = out[i * n + j] + s;                                              \
                    }                                                                                     \
                }                                                                                         \
            }                                                                                             \
        }                                                                                                 \
    }

/* 32-bit indices below n = 46340, as the reference (prk::get_max_matrix_size, prk_util.h:373-377);
 * 64-bit above. */
#define DEFINE_APPLY(P, PNAME, RR)                  \
    DEFINE_APPLY_T(P, PNAME, RR, int, _i32)         \
    DEFINE_APPLY_T(P, PNAME, RR, int64_t, _i64)     \
    static void apply_##PNAME##RR(const int64_t n, const int64_t t, const double* restrict in, double* restrict out) \
    {                                                                                                     \
        if (n <= 46340) apply_##PNAME##RR##_i32(n, t, in, out);                                          \
        else apply_##PNAME##RR##_i64(n, t, in, out);                                                      \
    }

DEFINE_APPLY(PRK_STAR, star, 1)
DEFINE_APPLY(PRK_STAR, star, 2)
DEFINE_APPLY(PRK_STAR, star, 3)
DEFINE_APPLY(PRK_STAR, star, 4)
DEFINE_APPLY(PRK_STAR, star, 5)
DEFINE_APPLY(PRK_GRID, grid, 1)
DEFINE_APPLY(PRK_GRID, grid, 2)
DEFINE_APPLY(PRK_GRID, grid, 3)
DEFINE_APPLY(PRK_GRID, grid, 4)
DEFINE_APPLY(PRK_GRID, grid, 5)

typedef void (*apply_fn)(const int64_t, const int64_t, const double* restrict, double* restrict);

/* The driver's dispatch switch (stencil-openmp.cc:154-171); NULL plays the part of nothing(). */
static apply_fn select_apply(int pattern, int R)
{
    static const apply_fn star[PRK_RMAX + 1] = {0, apply_star1, apply_star2, apply_star3, apply_star4, apply_star5};
    static const apply_fn grid[PRK_RMAX + 1] = {0, apply_grid1, apply_grid2, apply_grid3, apply_grid4, apply_grid5};
    if (R < 1 || R > PRK_RMAX) return 0;
    return pattern == PRK_GRID ? grid[R] : star[R];
}

static void add_one(const int64_t n, const int64_t t, double* restrict in)
{
    if (n <= 46340) {  /* 32-bit indices, as the reference */
        const int ni = (int)n, ti = (int)t;
        _Pragma("omp for collapse(2) schedule(static)")
        for (int it = 0; it < ni; it += ti)
            for (int jt = 0; jt < ni; jt += ti) {
                const int iend = (it + ti < ni) ? it + ti : ni;
                const int jend = (jt + ti < ni) ? jt + ti : ni;
                for (int i = it; i < iend; ++i) {
                    _Pragma("omp simd")
                    for (int j = jt; j < jend; ++j) in[i * ni + j] += 1.0;
                }
            }
        return;
    }
    _Pragma("omp for collapse(2) schedule(static)")
    for (int64_t it = 0; it < n; it += t)
        for (int64_t jt = 0; jt < n; jt += t) {
            const int64_t iend = (it + t < n) ? it + t : n;
            const int64_t jend = (jt + t < n) ? jt + t : n;
            for (int64_t i = it; i < iend; ++i) {
                _Pragma("omp simd")
                for (int64_t j = jt; j < jend; ++j) in[i * n + j] += 1.0;
            }
        }
}

static void init_grid(const int64_t n, const int64_t t, double* restrict in, double* restrict out)
{
    _Pragma("omp for collapse(2) schedule(static)")
    for (int64_t it = 0; it < n; it += t)
        for (int64_t jt = 0; jt < n; jt += t) {
            const int64_t iend = (it + t < n) ? it + t : n;
            const int64_t jend = (jt + t < n) ? jt + t : n;
            for (int64_t i = it; i < iend; ++i) {
                _Pragma("omp simd")
                for (int64_t j = jt; j < jend; ++j) {
                    in[i * n + j] = (double)(i + j);
                    out[i * n + j] = 0.0;
                }
            }
        }
}

static double now_s(void)
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

/* Argument checks of stencil-openmp.cc:94-143 (n without the 46340 cap: indices are 64-bit). */
static int check_args(int pattern, int R, int64_t n)
{
    if (pattern != PRK_STAR && pattern != PRK_GRID) return -1;
    if (n < 1) return -1;
    if (R < 1 || R > PRK_RMAX || 2 * (int64_t)R + 1 > n) return -1;
    return 0;
}

/* One application out += S(in) over the interior. Returns 0, or -1 on bad arguments. */
int prk_oracle_apply(int pattern, int R, int64_t n, int64_t tile, const double* in, double* out)
{
    if (check_args(pattern, R, n)) return -1;
    apply_fn f = select_apply(pattern, R);
    if (tile < 1 || tile > n) tile = n;
#pragma omp parallel
    f(n, tile, in, out);
    return 0;
}

/* in += 1.0 over the whole n x n (stencil-openmp.cc:208-218). */
int prk_oracle_add(int64_t n, int64_t tile, double* in)
{
    if (n < 1) return -1;
    if (tile < 1 || tile > n) tile = n;
#pragma omp parallel
    add_one(n, tile, in);
    return 0;
}

int prk_oracle_init(int64_t n, int64_t tile, double* in, double* out)
{
    if (n < 1) return -1;
    if (tile < 1 || tile > n) tile = n;
#pragma omp parallel
    init_grid(n, tile, in, out);
    return 0;
}

/* A whole PRK run as stencil-openmp.cc:182-223 does it: init, iterations+1 applications each
 * followed by in += 1, timer over iterations 1..K. *elapsed_s receives that time. */
int prk_oracle_run(int pattern, int R, int64_t n, int iterations, int64_t tile, double* in, double* out,
                   double* elapsed_s)
{
    if (check_args(pattern, R, n) || iterations < 1) return -1;
    apply_fn f = select_apply(pattern, R);
    if (tile < 1 || tile > n) tile = n;
    double t0 = 0.0, t1 = 0.0;
#pragma omp parallel
    {
        init_grid(n, tile, in, out);
        for (int iter = 0; iter <= iterations; ++iter) {
            if (iter == 1) {
#pragma omp barrier
#pragma omp master
                t0 = now_s();
            }
            f(n, tile, in, out);
            add_one(n, tile, in);
        }
#pragma omp barrier
#pragma omp master
        t1 = now_s();
    }
    if (elapsed_s) *elapsed_s = t1 - t0;
    return 0;
}

/* Timed sample for the CPU baseline: `applications` passes of stencil + add over caller-owned,
 * already initialised arrays. Returns wall seconds for the whole sample. */
double prk_oracle_sample(int pattern, int R, int64_t n, int applications, int64_t tile, double* in, double* out)
{
    if (check_args(pattern, R, n) || applications < 1) return -1.0;
    apply_fn f = select_apply(pattern, R);
    if (tile < 1 || tile > n) tile = n;
    double t0 = 0.0, t1 = 0.0;
#pragma omp parallel
    {
#pragma omp barrier
#pragma omp master
        t0 = now_s();
        for (int a = 0; a < applications; ++a) {
            f(n, tile, in, out);
            add_one(n, tile, in);
        }
#pragma omp barrier
#pragma omp master
        t1 = now_s();
    }
    return t1 - t0;
}

/* Serial L1 norm over the interior in row-major order, divided by (n-2R)^2
 * (stencil.cc:197-204; the OpenMP driver's reduction order is unspecified). */
double prk_oracle_norm(int R, int64_t n, const double* out)
{
    double norm = 0.0;
    for (int64_t i = R; i < n - R; ++i)
        for (int64_t j = R; j < n - R; ++j) norm += fabs(out[i * n + j]);
    return norm / ((double)(n - 2 * R) * (double)(n - 2 * R));
}

/* One application out += S(in) on a row slab of an n x n grid: in and out hold the grid rows
 * [first, first + nrows) with row stride n, and the points updated are the interior points of the
 * grid rows [row_begin, row_end) (which must lie inside the held rows, with R more either side
 * wherever the grid has them). Each point in the generator's strict order, as prk_oracle_apply: the
 * ranks of MPI1/Stencil/stencil.c:406-420 apply the stencil to their own block the same way.
 * Returns 0, or -1 on bad arguments. */
int prk_oracle_apply_rows(int pattern, int R, int64_t n, int64_t first, int64_t nrows, int64_t row_begin,
                          int64_t row_end, const double* in, double* out)
{
    if (check_args(pattern, R, n)) return -1;
    if (first < 0 || nrows < 1 || first + nrows > n || row_begin < first || row_end > first + nrows || row_begin > row_end)
        return -1;
    const int64_t lo = row_begin > R ? row_begin : R, hi = row_end < n - R ? row_end : n - R;
    if (lo < hi && (lo - R < first || hi + R > first + nrows)) return -1; /* the halo must be held */
    int dc[128], dr[128];
    double w[128];
    const int taps = prk_oracle_taps(pattern, R, dc, dr, w);
    for (int64_t i = lo; i < hi; ++i) {
        const double* row = in + (i - first) * n;
        for (int64_t j = R; j < n - R; ++j) {
            double s = 0.0;
            for (int q = 0; q < taps; ++q) {
                const double p = row[dr[q] * n + j + dc[q]] * w[q];
                s = (q == 0) ? p : s + p;
            }
            out[(i - first) * n + j] = out[(i - first) * n + j] + s;
        }
    }
    return 0;
}

/* out(i,j) after `applications` applications of a PRK run, computed for one interior point
 * without a grid: in_k(i,j) = i+j+k is exact in binary64 below 2^53, so the reference's value is
 * the left-to-right evaluation of the generated expression on those integers. Works for any n. */
double prk_oracle_point(int pattern, int R, int64_t n, int applications, int64_t i, int64_t j)
{
    (void)n;
    int dc[128], dr[128];
    double w[128];
    int taps = prk_oracle_taps(pattern, R, dc, dr, w);
    double out = 0.0;
    for (int k = 0; k < applications; ++k) {
        double s = 0.0;
        for (int q = 0; q < taps; ++q) {
            double v = (double)((i + dr[q]) + (j + dc[q]) + (int64_t)k);
            double p = v * w[q];
            s = (q == 0) ? p : s + p;
        }
        out = out + s;
    }
    return out;
}

/* PRK flop count (stencil-openmp.cc:254-255): (2*stencil_size+1)*(n-2R)^2, stencil_size = 4R+1
 * for star and (2R+1)^2 for grid. */
double prk_oracle_flops(int pattern, int R, int64_t n)
{
    double size = pattern == PRK_STAR ? 4.0 * R + 1.0 : (2.0 * R + 1.0) * (2.0 * R + 1.0);
    double act = (double)(n - 2 * R) * (double)(n - 2 * R);
    return (2.0 * size + 1.0) * act;
}

int prk_oracle_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
