// Generic stencil kernels: any n, any 8-byte-aligned buffers. Each CTA stages a TH x TW tile of
// `in` plus its R-wide halo in shared memory with coalesced loads, then every thread evaluates its
// points from shared memory: in_next = in + 1 over the tile (the fused sweep) and out += S(in) over
// the tile's part of the interior. Also the in += 1 pass, the initialisation and the L1 norm.
#include <type_traits>

#include "prk_arith.cuh"
#include "prk_internal.cuh"

namespace prk {
namespace {

constexpr int GEN_TW = 64;
constexpr int GEN_TH = 16;
constexpr int GEN_THREADS = 256;

template <int P, int R, int DT>
__global__ void __launch_bounds__(GEN_THREADS)
    k_stencil_generic(int64_t n, const void* __restrict__ in_v, void* __restrict__ in_next_v, void* __restrict__ out_v)
{
    using T = std::conditional_t<DT == FP64, double, float>;
    constexpr int SW = GEN_TW + 2 * R;
    constexpr int SH = GEN_TH + 2 * R;
    __shared__ T s[SH * SW];

    const T* __restrict__ in = static_cast<const T*>(in_v);
    T* __restrict__ in_next = static_cast<T*>(in_next_v);
    const int64_t i0 = static_cast<int64_t>(blockIdx.y) * GEN_TH;
    const int64_t j0 = static_cast<int64_t>(blockIdx.x) * GEN_TW;

    for (int idx = threadIdx.x; idx < SH * SW; idx += GEN_THREADS) {
        const int r = idx / SW, c = idx - r * SW;
        const int64_t gi = i0 - R + r, gj = j0 - R + c;
        T v = T(0);
        if (gi >= 0 && gi < n && gj >= 0 && gj < n) v = in[gi * n + gj];
        s[idx] = v;
    }
    __syncthreads();

    const int c = threadIdx.x % GEN_TW;
    for (int r = threadIdx.x / GEN_TW; r < GEN_TH; r += GEN_THREADS / GEN_TW) {
        const int64_t gi = i0 + r, gj = j0 + c;
        if (gi >= n || gj >= n) continue;
        const T* sp = s + (r + R) * SW + (c + R);
        if (in_next) {
            if constexpr (DT == FP64)
                in_next[gi * n + gj] = inc_exact(*sp);
            else
                in_next[gi * n + gj] = __fadd_rn(*sp, 1.0f);
        }
        if (gi >= R && gi < n - R && gj >= R && gj < n - R) {
            if constexpr (DT == FP64) {
                double* out = static_cast<double*>(out_v);
                out[gi * n + gj] = __dadd_rn(out[gi * n + gj], fp64_point<P, R>(sp, SW));
            } else {
                float2* out = static_cast<float2*>(out_v);
                float2 o = out[gi * n + gj];
                float sh, sl;
                fp32c_point<P, R>(sp, SW, sh, sl);
                df_add(o.x, o.y, sh, sl);
                out[gi * n + gj] = o;
            }
        }
    }
}

using GenericFn = void (*)(int64_t, const void*, void*, void*);

template <int DT>
GenericFn pick_generic(int pattern, int R)
{
    if (pattern == STAR) {
        switch (R) {
        case 1: return k_stencil_generic<STAR, 1, DT>;
        case 2: return k_stencil_generic<STAR, 2, DT>;
        case 3: return k_stencil_generic<STAR, 3, DT>;
        case 4: return k_stencil_generic<STAR, 4, DT>;
        case 5: return k_stencil_generic<STAR, 5, DT>;
        }
    } else {
        switch (R) {
        case 1: return k_stencil_generic<GRID, 1, DT>;
        case 2: return k_stencil_generic<GRID, 2, DT>;
        case 3: return k_stencil_generic<GRID, 3, DT>;
        case 4: return k_stencil_generic<GRID, 4, DT>;
        case 5: return k_stencil_generic<GRID, 5, DT>;
        }
    }
    return nullptr;
}

template <int DT>
__global__ void k_add(int64_t total, void* in_v)
{
    using T = std::conditional_t<DT == FP64, double, float>;
    T* in = static_cast<T*>(in_v);
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < total; k += stride) {
        if constexpr (DT == FP64)
            in[k] = inc_exact(in[k]);
        else
            in[k] = __fadd_rn(in[k], 1.0f);
    }
}

template <int DT>
__global__ void k_init(int64_t n, void* in_v, void* out_v)
{
    using T = std::conditional_t<DT == FP64, double, float>;
    T* in = static_cast<T*>(in_v);
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
            in[i * n + j] = static_cast<T>(i + j);
            if constexpr (DT == FP64)
                static_cast<double*>(out_v)[i * n + j] = 0.0;
            else
                static_cast<float2*>(out_v)[i * n + j] = make_float2(0.0f, 0.0f);
        }
    }
    (void)stride;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum in a fixed order (warp shuffles, then warp 0 over the warp totals).
template <int THREADS>
__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double warp_tot[THREADS / 32];
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) warp_tot[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < THREADS / 32 ? warp_tot[threadIdx.x] : 0.0;
        t = warp_sum(t);
    }
    return t;  // valid in thread 0
}

constexpr int NORM_THREADS = 256;

// |d| as an unevaluated pair of floats h + l, from the binary64 encoding alone (the binary64 pipe
// runs conversions at its slow rate): h holds the top 24 bits of the significand and l the next 23,
// rounded on the bit below, so |(h + l) - |d|| <= 2^-47 |d|. Returns false, leaving h and l
// untouched, when d is zero or its exponent lies outside [2^-60, 2^77), where the pair's exponents
// would leave float's normal range; the caller adds such values in binary64.
__device__ __forceinline__ bool abs_as_float_pair(uint64_t b, float& h, float& l)
{
    const uint32_t hi = static_cast<uint32_t>(b >> 32) & 0x7FFFFFFFu, lo = static_cast<uint32_t>(b);
    const uint32_t e = hi >> 20;  // biased binary64 exponent
    if (e < 963u || e >= 1100u) return false;
    // h: same exponent (rebias by 1023 - 127 = 896), fraction bits 51..29
    h = __uint_as_float(((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
    // l: fraction bits 28..6, rounded half up on bit 5, as an integer x <= 2^23 worth
    // x * 2^(e - 1075 + 6): float(x) by the 2^23 magic number (exact; x = 2^23 carries into the
    // exponent field and still comes out exact), then scaled by that power of two (exact, normal for
    // e >= 963)
    const uint32_t xi = (((lo >> 5) & 0xFFFFFFu) + 1u) >> 1;
    const float x = __fsub_rn(__uint_as_float(0x4B000000u | xi), 8388608.0f);
    l = __fmul_rn(x, __uint_as_float((e - 1075u + 6u + 127u) << 23));
    return true;
}

// Per-block partial sums of |out| over the interior columns of array rows i_lo + blockIdx.x,
// i_lo + blockIdx.x + gridDim.x, ... below i_hi.
// Both forms accumulate per thread as a two-float sum (TwoSum on the high parts, the errors and the
// low parts into the low word) and widen to binary64 once per thread at the end: FP32C from its
// (hi, lo) words, FP64 from each |value| split into a float pair by abs_as_float_pair (relative
// error at most 2^-47 per value; values outside that range, zeros aside, go into a binary64 sum).
// Four columns per thread per trip keep four loads in flight. The order of every sum is fixed, so
// the result is deterministic.
template <int DT>
__global__ void __launch_bounds__(NORM_THREADS) k_norm_partial(int R, int64_t n, int64_t i_lo, int64_t i_hi,
                                                               const void* out_v, double* partial)
{
    double acc = 0.0;
    float ah = 0.0f, al = 0.0f;
    auto add_pair = [&](float h, float l) {
        float t, e;
        two_sum(ah, h, t, e);
        ah = t;
        al = __fadd_rn(al, __fadd_rn(e, l));
    };
    constexpr int U = 4;
    for (int64_t i = i_lo + blockIdx.x; i < i_hi; i += gridDim.x) {
        const int64_t end = n - R;
        for (int64_t j0 = R + threadIdx.x; j0 < end; j0 += U * NORM_THREADS) {
            if constexpr (DT == FP64) {
                const uint64_t* row = static_cast<const uint64_t*>(out_v) + i * n;
                uint64_t b[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int64_t j = j0 + u * NORM_THREADS;
                    b[u] = j < end ? row[j] : 0ull;
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    float h, l;
                    if (abs_as_float_pair(b[u], h, l))
                        add_pair(h, l);
                    else if ((b[u] << 1) != 0ull)
                        acc = __dadd_rn(acc, fabs(__longlong_as_double(static_cast<long long>(b[u]))));
                }
            } else {
                const float2* row = static_cast<const float2*>(out_v) + i * n;
                float2 o[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int64_t j = j0 + u * NORM_THREADS;
                    o[u] = j < end ? row[j] : make_float2(0.0f, 0.0f);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (o[u].x < 0.0f || (o[u].x == 0.0f && o[u].y < 0.0f)) {
                        o[u].x = -o[u].x;
                        o[u].y = -o[u].y;
                    }
                    add_pair(o[u].x, o[u].y);
                }
            }
        }
    }
    acc = __dadd_rn(acc, __dadd_rn(static_cast<double>(ah), static_cast<double>(al)));
    const double tot = block_sum<NORM_THREADS>(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// Binary64 add throughput: every thread runs 8 independent chains of `iters` adds. The sum is
// stored only when it equals a value the chains cannot reach, which keeps the adds live.
__global__ void __launch_bounds__(256) k_dadd_probe(double* sink, double step, int iters)
{
    double a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = static_cast<double>(threadIdx.x) + 0.125 * k;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = __dadd_rn(a[k], step);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s = __dadd_rn(s, a[k]);
    if (s == -1.0) sink[0] = s;
}

// Sum of the partials in a fixed order, scaled by 1/(n-2R)^2.
__global__ void __launch_bounds__(NORM_THREADS) k_norm_final(const double* partial, int count, double active,
                                                             double* result)
{
    double acc = 0.0;
    for (int k = threadIdx.x; k < count; k += NORM_THREADS) acc += partial[k];
    const double tot = block_sum<NORM_THREADS>(acc);
    if (threadIdx.x == 0) *result = tot / active;
}

int grid_for(int64_t work, int threads, int cap)
{
    int64_t b = (work + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return static_cast<int>(b);
}

}  // namespace

cudaError_t launch_stencil_generic(const StencilCall& c)
{
    GenericFn f = c.dtype == FP64 ? pick_generic<FP64>(c.pattern, c.R) : pick_generic<FP32C>(c.pattern, c.R);
    if (!f) return cudaErrorInvalidValue;
    const dim3 grid(static_cast<unsigned>((c.n + GEN_TW - 1) / GEN_TW), static_cast<unsigned>((c.n + GEN_TH - 1) / GEN_TH));
    f<<<grid, GEN_THREADS, 0, c.stream>>>(c.n, c.in, c.in_next, c.out);
    return cudaGetLastError();
}

cudaError_t launch_add(int64_t n, int dtype, void* in, cudaStream_t s)
{
    const int64_t total = n * n;
    const int blocks = grid_for(total, 256, 152 * 32);
    if (dtype == FP64)
        k_add<FP64><<<blocks, 256, 0, s>>>(total, in);
    else
        k_add<FP32C><<<blocks, 256, 0, s>>>(total, in);
    return cudaGetLastError();
}

cudaError_t launch_init(int64_t n, int dtype, void* in, void* out, cudaStream_t s)
{
    const int blocks = static_cast<int>(n < 65535 ? n : 65535);
    if (dtype == FP64)
        k_init<FP64><<<blocks, 256, 0, s>>>(n, in, out);
    else
        k_init<FP32C><<<blocks, 256, 0, s>>>(n, in, out);
    return cudaGetLastError();
}

cudaError_t launch_dadd_probe(double* sink, int blocks, int iters, double step, cudaStream_t s)
{
    k_dadd_probe<<<blocks, 256, 0, s>>>(sink, step, iters);
    return cudaGetLastError();
}

cudaError_t launch_norm_rows(int R, int64_t n, int dtype, const void* out, int64_t i_lo, int64_t i_hi, double divisor,
                             double* partial, double* result_dev, cudaStream_t s)
{
    const int64_t rows = i_hi > i_lo ? i_hi - i_lo : 0;
    const int blocks = static_cast<int>(rows < NORM_BLOCKS ? rows : NORM_BLOCKS);
    if (blocks > 0) {
        if (dtype == FP64)
            k_norm_partial<FP64><<<blocks, NORM_THREADS, 0, s>>>(R, n, i_lo, i_hi, out, partial);
        else
            k_norm_partial<FP32C><<<blocks, NORM_THREADS, 0, s>>>(R, n, i_lo, i_hi, out, partial);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    k_norm_final<<<1, NORM_THREADS, 0, s>>>(partial, blocks, divisor, result_dev);
    return cudaGetLastError();
}

cudaError_t launch_norm(int R, int64_t n, int dtype, const void* out, double* partial, double* result_dev, cudaStream_t s)
{
    const double active = static_cast<double>(n - 2 * R) * static_cast<double>(n - 2 * R);
    return launch_norm_rows(R, n, dtype, out, R, n - R, active, partial, result_dev, s);
}

}  // namespace prk
