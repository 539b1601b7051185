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

// Per-block partial sums of |out| over interior rows blockIdx.x, blockIdx.x + gridDim.x, ...
// FP64: binary64 accumulation. FP32C: each |hi+lo| is accumulated as a two-float sum per thread and
// widened to binary64 once at the end.
template <int DT>
__global__ void __launch_bounds__(NORM_THREADS) k_norm_partial(int R, int64_t n, const void* out_v, double* partial)
{
    double acc = 0.0;
    float ah = 0.0f, al = 0.0f;
    for (int64_t i = R + blockIdx.x; i < n - R; i += gridDim.x) {
        for (int64_t j = R + threadIdx.x; j < n - R; j += NORM_THREADS) {
            if constexpr (DT == FP64) {
                acc = __dadd_rn(acc, fabs(static_cast<const double*>(out_v)[i * n + j]));
            } else {
                float2 o = static_cast<const float2*>(out_v)[i * n + j];
                if (o.x < 0.0f || (o.x == 0.0f && o.y < 0.0f)) {
                    o.x = -o.x;
                    o.y = -o.y;
                }
                float t, e;
                two_sum(ah, o.x, t, e);
                ah = t;
                al = __fadd_rn(al, __fadd_rn(e, o.y));
            }
        }
    }
    if constexpr (DT != FP64) acc = static_cast<double>(ah) + static_cast<double>(al);
    const double tot = block_sum<NORM_THREADS>(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = tot;
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

cudaError_t launch_norm(int R, int64_t n, int dtype, const void* out, double* partial, double* result_dev, cudaStream_t s)
{
    const int64_t rows = n - 2 * R;
    const int blocks = static_cast<int>(rows < NORM_BLOCKS ? rows : NORM_BLOCKS);
    if (dtype == FP64)
        k_norm_partial<FP64><<<blocks, NORM_THREADS, 0, s>>>(R, n, out, partial);
    else
        k_norm_partial<FP32C><<<blocks, NORM_THREADS, 0, s>>>(R, n, out, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const double active = static_cast<double>(rows) * static_cast<double>(rows);
    k_norm_final<<<1, NORM_THREADS, 0, s>>>(partial, blocks, active, result_dev);
    return cudaGetLastError();
}

}  // namespace prk
