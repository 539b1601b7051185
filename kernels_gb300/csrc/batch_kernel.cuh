// The batched stencil kernel: many independent grids of uneven n, mixed radius and pattern in one
// persistent launch.
//
// The work list of a launch is every tile of every grid in the batch. CTAs pop work items from a
// device queue (one atomic counter per launch) until the list is exhausted, so grids of very
// different sizes balance across the SMs. An item is mapped to its grid by a binary search over the
// grids' tile offsets. The grid's `in` tile and halo are staged in shared memory with coalesced
// loads, zero outside the grid, because batch grids have arbitrary n and alignment. The tile is then
// evaluated by the same code as the TMA kernels (stencil_tile.cuh), with the pattern and radius
// picked per item by a switch.
//
// Every launch advances all grids of the launch by STEPS applications (temporal depth; STEPS = 0
// takes `depth` at run time, for a whole run in one launch), ping-ponging between each grid's two
// `in` buffers; `parity` says which one holds the current `in`.
#pragma once

#include "stencil_tile.cuh"

namespace prk {
namespace batch {

// Device-side descriptor of one grid (64 bytes).
struct GridDesc {
    int64_t n;
    void* in[2];
    void* out;
    int pattern;
    int R;
    int tiles_x;
    int vec_ok;  // 16-byte-aligned buffers and n a multiple of the vector width
    int64_t tiles;
};

template <int DT>
constexpr int max_in_bytes()
{
    int m = 0;
#define PRK_MAXB(RR) m = tile::Geo<DT, RR>::IN_BYTES > m ? tile::Geo<DT, RR>::IN_BYTES : m;
    PRK_MAXB(1) PRK_MAXB(2) PRK_MAXB(3) PRK_MAXB(4) PRK_MAXB(5)
#undef PRK_MAXB
    return m;
}

template <int DT>
struct Layout {
    static constexpr int RED_OFF = (max_in_bytes<DT>() + 127) / 128 * 128;
    static constexpr int SMEM = RED_OFF + tile::WARPS * 8;
};

// Stage the `in` tile at (i0, j0) with its halo in shared memory: coalesced plain loads, zero
// outside the arrays (nr rows of n columns), all loads issued before the first shared-memory store. Thread t takes elements
// t, t + THREADS, ... of the row-major tile; its row, column and grid offset advance by constants
// from one element to the next (one division per thread, none per element).
template <int R, int DT>
__device__ __forceinline__ void stage_tile(unsigned char* smem, const void* in_v, int64_t n, int64_t nr, int64_t i0,
                                           int64_t j0)
{
    using G = tile::Geo<DT, R>;
    using T = typename tile::Cfg<DT>::T;
    constexpr int PER = (G::ELEMS + tile::THREADS - 1) / tile::THREADS;
    constexpr int DR = tile::THREADS / G::SW, DC = tile::THREADS % G::SW;
    const T* __restrict__ in = static_cast<const T*>(in_v);
    T* s_in = reinterpret_cast<T*>(smem);
    const uint32_t un = static_cast<uint32_t>(n), unr = static_cast<uint32_t>(nr);  // n, nr <= NMAX < 2^31
    int r = threadIdx.x / G::SW, c = threadIdx.x - (threadIdx.x / G::SW) * G::SW;
    int gi = static_cast<int>(i0) - R + r, gj = static_cast<int>(j0) - G::RA + c;
    int64_t off = static_cast<int64_t>(gi) * n + gj;
    T v[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {  // all loads first, then the shared-memory stores
        const int idx = threadIdx.x + q * tile::THREADS;
        const bool ok = (q + 1) * tile::THREADS <= G::ELEMS || idx < G::ELEMS;
        v[q] = (ok && static_cast<uint32_t>(gi) < unr && static_cast<uint32_t>(gj) < un) ? in[off] : T(0);
        c += DC;
        gi += DR;
        gj += DC;
        off += DR * n + DC;
        if (c >= G::SW) {
            c -= G::SW;
            gi += 1;
            gj -= G::SW;
            off += n - G::SW;
        }
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int idx = threadIdx.x + q * tile::THREADS;
        if (idx < G::ELEMS) s_in[idx] = v[q];
    }
    __syncthreads();
}

// One work item: load the tile of grid g at `parity`, then evaluate it.
template <int P, int R, int DT, int STEPS>
__device__ __forceinline__ void item(unsigned char* smem, int* s_red, const GridDesc& g, int64_t t, int parity,
                                     int depth)
{
    using C = tile::Cfg<DT>;
    const int64_t n = g.n;
    const int64_t i0 = (t / g.tiles_x) * C::TH;
    const int64_t j0 = (t % g.tiles_x) * C::TW;
    stage_tile<R, DT>(smem, g.in[parity], n, n, i0, j0);
    tile::process_tile<P, R, DT, STEPS, tile::OUT_HBM>(smem, s_red, i0, j0, n, tile::tile_has_out(i0, j0, n, R, C::TW, C::TH),
                                               g.in[parity ^ 1], g.out, g.vec_ok != 0, depth, 0, n);
}

template <int DT, int STEPS>
__device__ __forceinline__ void dispatch(unsigned char* smem, int* s_red, const GridDesc& g, int64_t t, int parity,
                                         int depth)
{
#define PRK_ITEM(PP, RR) \
    case RR: item<PP, RR, DT, STEPS>(smem, s_red, g, t, parity, depth); break;
    if (g.pattern == STAR) {
        switch (g.R) { PRK_ITEM(STAR, 1) PRK_ITEM(STAR, 2) PRK_ITEM(STAR, 3) PRK_ITEM(STAR, 4) PRK_ITEM(STAR, 5) }
    } else {
        switch (g.R) { PRK_ITEM(GRID, 1) PRK_ITEM(GRID, 2) PRK_ITEM(GRID, 3) PRK_ITEM(GRID, 4) PRK_ITEM(GRID, 5) }
    }
#undef PRK_ITEM
}

template <int DT, int STEPS>
__global__ void __launch_bounds__(tile::THREADS, 2)
    k_batch(const GridDesc* __restrict__ grids, const int64_t* __restrict__ tile_off, int ngrids, int64_t total,
            unsigned long long* __restrict__ queue, int parity, int depth)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ long long s_item;
    int* s_red = reinterpret_cast<int*>(smem + Layout<DT>::RED_OFF);
    for (;;) {
        if (threadIdx.x == 0) s_item = static_cast<long long>(atomicAdd(queue, 1ull));
        __syncthreads();
        const long long it = s_item;
        if (it >= total) break;
        int lo = 0, hi = ngrids;  // tile_off[lo] <= it < tile_off[lo + 1]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (tile_off[mid] <= it) lo = mid;
            else hi = mid;
        }
        const GridDesc g = grids[lo];
        dispatch<DT, STEPS>(smem, s_red, g, it - tile_off[lo], parity, depth);
        __syncthreads();  // shared memory and s_item are reused by the next item
    }
}

struct Launch {
    const GridDesc* grids;
    const int64_t* tile_off;
    int ngrids;
    int64_t total;
    unsigned long long* queue;
    int parity;
    int ctas;  // persistent CTAs
    cudaStream_t stream;
    int depth;  // applications of a run-time-depth launch (STEPS = 0)
};

template <int DT, int STEPS>
cudaError_t launch(const Launch& L)
{
    if (cudaError_t e = cudaFuncSetAttribute(k_batch<DT, STEPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, Layout<DT>::SMEM))
        return e;
    if (STEPS == 0 && L.depth < 1) return cudaErrorInvalidValue;
    k_batch<DT, STEPS><<<L.ctas, tile::THREADS, Layout<DT>::SMEM, L.stream>>>(L.grids, L.tile_off, L.ngrids, L.total,
                                                                             L.queue, L.parity, L.depth);
    return cudaGetLastError();
}

// Resident CTAs per SM of k_batch<DT, STEPS> (occupancy query; 0 on failure).
template <int DT, int STEPS>
int ctas_per_sm()
{
    int b = 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch<DT, STEPS>, tile::THREADS, Layout<DT>::SMEM) == cudaSuccess
               ? b : 0;
}

// Each (form, depth) pair is instantiated in one translation unit (batch_fp64*.cu, batch_fp32c*.cu)
// so that the build compiles them in parallel; the dispatching units declare them with this.
#define PRK_BATCH_EXTERN(DT, S)                                  \
    extern template cudaError_t launch<DT, S>(const Launch& L); \
    extern template int ctas_per_sm<DT, S>();
#define PRK_BATCH_INSTANTIATE(DT, S)                      \
    template cudaError_t launch<DT, S>(const Launch& L); \
    template int ctas_per_sm<DT, S>();

template <int DT>
cudaError_t launch_depth(int steps, const Launch& L)
{
    switch (steps) {
    case 1: return launch<DT, 1>(L);
    case 2: return launch<DT, 2>(L);
    case 4: return launch<DT, 4>(L);
    case 8: return launch<DT, 8>(L);
    case 0: return launch<DT, 0>(L);
    }
    return cudaErrorInvalidValue;
}

template <int DT>
int ctas_per_sm_depth(int steps)
{
    switch (steps) {
    case 1: return ctas_per_sm<DT, 1>();
    case 2: return ctas_per_sm<DT, 2>();
    case 4: return ctas_per_sm<DT, 4>();
    case 8: return ctas_per_sm<DT, 8>();
    case 0: return ctas_per_sm<DT, 0>();
    }
    return 0;
}

// Per-form entry points (batch_fp64.cu, batch_fp32c.cu).
cudaError_t launch_fp64(int steps, const Launch& L);
cudaError_t launch_fp32c(int steps, const Launch& L);
// Resident CTAs per SM of the batched kernel at a depth (occupancy query; 0 on failure).
int ctas_per_sm_fp64(int steps);
int ctas_per_sm_fp32c(int steps);

}  // namespace batch
}  // namespace prk
