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

// Kernel families: the stencils one instantiation of the batched kernel evaluates, so that no kernel
// carries the code and registers of stencils it does not run. FP32C: the star stencils, and the grid
// stencils. FP64: the power-of-two stencils (star R=1,2 and grid R=1, the certified exact routes),
// and each stencil with other weights on its own (the table route).
constexpr int FAM_F32_STAR = 0;
constexpr int FAM_F32_GRID = 1;
constexpr int FAM_POW2 = 2;
__host__ __device__ constexpr int fam_one(int P, int R) { return 16 + 8 * P + R; }

__host__ __device__ constexpr bool in_family(int fam, int P, int R, int DT)
{
    if (fam == FAM_F32_STAR) return DT == FP32C && P == STAR;
    if (fam == FAM_F32_GRID) return DT == FP32C && P == GRID;
    if (fam == FAM_POW2) return DT == FP64 && pow2_weights(P, R);
    return DT == FP64 && fam == fam_one(P, R) && !pow2_weights(P, R);
}

// The family that evaluates a grid of (pattern, R) in storage form dtype.
__host__ __device__ constexpr int family_of(int dtype, int P, int R)
{
    return dtype == FP32C ? (P == STAR ? FAM_F32_STAR : FAM_F32_GRID) : (pow2_weights(P, R) ? FAM_POW2 : fam_one(P, R));
}

template <int DT, int FAM>
constexpr int max_in_bytes()
{
    int m = 0;
    for (int P = 0; P < 2; ++P) {
#define PRK_MAXB(RR) \
    if (in_family(FAM, P, RR, DT) && tile::Geo<DT, RR>::IN_BYTES > m) m = tile::Geo<DT, RR>::IN_BYTES;
        PRK_MAXB(1) PRK_MAXB(2) PRK_MAXB(3) PRK_MAXB(4) PRK_MAXB(5)
#undef PRK_MAXB
    }
    return m;
}

template <int DT, int FAM>
constexpr int max_table_bytes()
{
    int m = 0;
#define PRK_MAXT(PP, RR) \
    if (in_family(FAM, PP, RR, DT) && tile::table_bytes<PP, RR, DT>() > m) m = tile::table_bytes<PP, RR, DT>();
    PRK_MAXT(STAR, 1) PRK_MAXT(STAR, 2) PRK_MAXT(STAR, 3) PRK_MAXT(STAR, 4) PRK_MAXT(STAR, 5)
    PRK_MAXT(GRID, 1) PRK_MAXT(GRID, 2) PRK_MAXT(GRID, 3) PRK_MAXT(GRID, 4) PRK_MAXT(GRID, 5)
#undef PRK_MAXT
    return m;
}

// Shared memory: the staged `in` tile, the reduction words, and the table route's product tables
// followed by its out area (tile::table_tile).
template <int DT, int FAM>
struct Layout {
    static constexpr int RED_OFF = (max_in_bytes<DT, FAM>() + 127) / 128 * 128;
    static constexpr int TBL_OFF = (RED_OFF + tile::WARPS * 8 + 15) / 16 * 16;
    static constexpr int SMEM =
        TBL_OFF + max_table_bytes<DT, FAM>() + (max_table_bytes<DT, FAM>() > 0 ? tile::table_out_bytes() : 0);
    static_assert(SMEM <= tile::SMEM_PER_CTA_MAX, "the tile and its tables must fit in shared memory");
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

// One work item: load the tile of grid g at `parity`, then evaluate it. tbl: the table area.
template <int P, int R, int DT, int STEPS>
__device__ __forceinline__ void item(unsigned char* smem, int* s_red, const GridDesc& g, int64_t t, int parity,
                                     int depth, unsigned char* tbl)
{
    using C = tile::Cfg<DT>;
    const int64_t n = g.n;
    const int64_t i0 = (t / g.tiles_x) * C::TH;
    const int64_t j0 = (t % g.tiles_x) * C::TW;
    // the two in buffers picked without indexing g.in by a run-time value (which would put g in
    // local memory)
    void* const in_cur = parity ? g.in[1] : g.in[0];
    void* const in_nxt = parity ? g.in[0] : g.in[1];
    stage_tile<R, DT>(smem, in_cur, n, n, i0, j0);
    tile::process_tile<P, R, DT, STEPS, tile::OUT_HBM>(smem, s_red, i0, j0, n, tile::tile_has_out(i0, j0, n, R, C::TW, C::TH),
                                               in_nxt, g.out, g.vec_ok != 0, depth, 0, n,
                                               tile::table_route<P, R, DT>() ? tbl : nullptr);
}

template <int DT, int STEPS, int FAM>
__device__ __forceinline__ void dispatch(unsigned char* smem, int* s_red, const GridDesc& g, int64_t t, int parity,
                                         int depth, unsigned char* tbl)
{
#define PRK_ITEM(PP, RR)                                                                  \
    case RR:                                                                              \
        if constexpr (in_family(FAM, PP, RR, DT)) item<PP, RR, DT, STEPS>(smem, s_red, g, t, parity, depth, tbl); \
        break;
    if (g.pattern == STAR) {
        switch (g.R) { PRK_ITEM(STAR, 1) PRK_ITEM(STAR, 2) PRK_ITEM(STAR, 3) PRK_ITEM(STAR, 4) PRK_ITEM(STAR, 5) }
    } else {
        switch (g.R) { PRK_ITEM(GRID, 1) PRK_ITEM(GRID, 2) PRK_ITEM(GRID, 3) PRK_ITEM(GRID, 4) PRK_ITEM(GRID, 5) }
    }
#undef PRK_ITEM
}

template <int DT, int STEPS, int FAM>
__global__ void __launch_bounds__(tile::THREADS, 2)
    k_batch(const GridDesc* __restrict__ grids, const int64_t* __restrict__ tile_off, int ngrids, int64_t total,
            unsigned long long* __restrict__ queue, int parity, int depth)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ long long s_item;
    int* s_red = reinterpret_cast<int*>(smem + Layout<DT, FAM>::RED_OFF);
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
        dispatch<DT, STEPS, FAM>(smem, s_red, g, it - tile_off[lo], parity, depth, smem + Layout<DT, FAM>::TBL_OFF);
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

template <int DT, int STEPS, int FAM>
cudaError_t launch(const Launch& L)
{
    constexpr int SM = Layout<DT, FAM>::SMEM;
    if (cudaError_t e = cudaFuncSetAttribute(k_batch<DT, STEPS, FAM>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM))
        return e;
    if (STEPS == 0 && L.depth < 1) return cudaErrorInvalidValue;
    k_batch<DT, STEPS, FAM><<<L.ctas, tile::THREADS, SM, L.stream>>>(L.grids, L.tile_off, L.ngrids, L.total, L.queue,
                                                                      L.parity, L.depth);
    return cudaGetLastError();
}

// Resident CTAs per SM of k_batch<DT, STEPS, FAM> (occupancy query; 0 on failure).
template <int DT, int STEPS, int FAM>
int ctas_per_sm()
{
    constexpr int SM = Layout<DT, FAM>::SMEM;
    int b = 0;
    if (cudaFuncSetAttribute(k_batch<DT, STEPS, FAM>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM) != cudaSuccess) return 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch<DT, STEPS, FAM>, tile::THREADS, SM) == cudaSuccess
               ? b : 0;
}

template <int DT, int FAM>
cudaError_t launch_depth(int steps, const Launch& L)
{
    switch (steps) {
    case 1: return launch<DT, 1, FAM>(L);
    case 2: return launch<DT, 2, FAM>(L);
    case 4: return launch<DT, 4, FAM>(L);
    case 8: return launch<DT, 8, FAM>(L);
    case 0: return launch<DT, 0, FAM>(L);
    }
    return cudaErrorInvalidValue;
}

template <int DT, int FAM>
int ctas_per_sm_depth(int steps)
{
    switch (steps) {
    case 1: return ctas_per_sm<DT, 1, FAM>();
    case 2: return ctas_per_sm<DT, 2, FAM>();
    case 4: return ctas_per_sm<DT, 4, FAM>();
    case 8: return ctas_per_sm<DT, 8, FAM>();
    case 0: return ctas_per_sm<DT, 0, FAM>();
    }
    return 0;
}

// Per-family entry points, one translation unit each so that the build compiles them in parallel:
// batch_fp64_pow2.cu, batch_fp64_strict_*.cu (one per stencil with other weights),
// batch_fp32c_star.cu and batch_fp32c_grid.cu.
cudaError_t launch_fp64_pow2(int steps, const Launch& L);
int ctas_per_sm_fp64_pow2(int steps);
#define PRK_BATCH_STRICT_DECL(PN, RR)                                 \
    cudaError_t launch_fp64_##PN##RR(int steps, const Launch& L); \
    int ctas_per_sm_fp64_##PN##RR(int steps);
PRK_BATCH_STRICT_DECL(star, 3)
PRK_BATCH_STRICT_DECL(star, 4)
PRK_BATCH_STRICT_DECL(star, 5)
PRK_BATCH_STRICT_DECL(grid, 2)
PRK_BATCH_STRICT_DECL(grid, 3)
PRK_BATCH_STRICT_DECL(grid, 4)
PRK_BATCH_STRICT_DECL(grid, 5)
#undef PRK_BATCH_STRICT_DECL

cudaError_t launch_fp32c_star(int steps, const Launch& L);
int ctas_per_sm_fp32c_star(int steps);
cudaError_t launch_fp32c_grid(int steps, const Launch& L);
int ctas_per_sm_fp32c_grid(int steps);

// Dispatch by family (host side): a grid's family as family_of gives it.
cudaError_t launch_family(int dtype, int fam, int steps, const Launch& L);
int ctas_per_sm_family(int dtype, int fam, int steps);

}  // namespace batch
}  // namespace prk
