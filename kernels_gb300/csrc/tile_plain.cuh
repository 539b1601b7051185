// The tile kernel for shapes a tensor map cannot describe: n not a multiple of the vector width
// (rows not 16-byte multiples) or buffers that are not 16-byte aligned.
//
// One CTA per tile, as in the TMA kernel, so that several tiles per SM are in flight at once. The
// `in` tile and its halo are staged in shared memory (zero outside the grid) with coalesced plain
// loads, or, with the `out` tile, by per-element asynchronous copies (cp.async) for the stencils
// that take the table route, and the tile is evaluated by the same code as the TMA and batched
// kernels (stencil_tile.cuh): the same exact routes, the same certification.
// STEPS = 1 is one application per launch; STEPS = 0 takes the number of applications at run time
// (any temporal depth, or a whole run).
#pragma once

#include "batch_kernel.cuh"

namespace prk {
namespace plain {

// Shared memory. The stencils that take the table route (tile::table_route): the TMA kernel's
// layout (the `in` tile with its halo, the `out` tile, the certification's reduction words) and the
// product tables. The others: the `in` tile and the reduction words.
template <int P, int DT, int R>
struct Smem {
    using G = tile::Geo<DT, R>;
    static constexpr bool TBL = tile::table_route<P, R, DT>();
    static constexpr int RED_OFF = TBL ? G::RED_OFF : (G::IN_BYTES + 127) / 128 * 128;
    static constexpr int TBL_OFF = tile::table_offset<DT, R, tile::TH_DEFAULT>();
    static constexpr int BYTES = TBL ? tile::tile_smem<P, R, DT, tile::TH_DEFAULT>() : RED_OFF + tile::WARPS * 8;
    static_assert(BYTES <= tile::SMEM_PER_CTA_MAX, "the tile and its tables must fit in shared memory");
};

// Resident CTAs per SM the register budget is cut for: the TMA kernel's (three tiles per SM for the
// table route), except for the FP64 power-of-two stencils at one application, whose out words are
// all requested ahead (tile::OUT_HBM_AHEAD) and which hold them in the registers of five CTAs per SM
// rather than spilling at six (n=16383, star R=2: 3585 GFLOP/s against 3449 without the early
// requests).
template <int P, int R, int DT, int STEPS>
constexpr int plain_min_blocks()
{
    constexpr int b = tile::min_blocks<P, R, DT, STEPS, tile::TH_DEFAULT>();
    return DT == FP64 && pow2_weights(P, R) && STEPS == 1 && b > 5 ? 5 : b;
}

// Stage the tile with asynchronous copies (cp.async), one element each: the `in` tile with its halo
// (SH rows of SW elements from array row i0 - R, column j0 - RA) and, when the tile has interior
// points, the `out` tile (TH rows of TW words from (i0, j0)), in the TMA kernel's layout; elements
// outside the arrays are written as zeros without a read. Every copy of the tile is in flight at
// once and none passes through registers; the thread then waits for its copies and the block
// meets at a barrier.
template <int R, int DT>
__device__ __forceinline__ void stage_async(unsigned char* smem, const void* in_v, const void* out_v, int64_t n,
                                            int64_t nr, int64_t i0, int64_t j0, bool has_out)
{
    using G = tile::Geo<DT, R>;
    using C = tile::Cfg<DT>;
    using T = typename C::T;
    constexpr int E = static_cast<int>(sizeof(T));
    constexpr int PER = (G::ELEMS + tile::THREADS - 1) / tile::THREADS;
    constexpr int DR = tile::THREADS / G::SW, DC = tile::THREADS % G::SW;
    const T* __restrict__ in = static_cast<const T*>(in_v);
    T* s_in = reinterpret_cast<T*>(smem);
    const uint32_t un = static_cast<uint32_t>(n), unr = static_cast<uint32_t>(nr);  // n, nr <= NMAX < 2^31
    int c = threadIdx.x - (threadIdx.x / G::SW) * G::SW;
    int gi = static_cast<int>(i0) - R + static_cast<int>(threadIdx.x / G::SW), gj = static_cast<int>(j0) - G::RA + c;
    int64_t off = static_cast<int64_t>(gi) * n + gj;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int idx = threadIdx.x + q * tile::THREADS;
        if ((q + 1) * tile::THREADS <= G::ELEMS || idx < G::ELEMS) {
            const bool ok = static_cast<uint32_t>(gi) < unr && static_cast<uint32_t>(gj) < un;
            cp_async<E>(s_in + idx, ok ? in + off : in, ok ? E : 0);
        }
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
    if (has_out) {
        static_assert((C::TW & (C::TW - 1)) == 0 && (C::TW * C::TH) % tile::THREADS == 0, "out tile layout");
        const uint64_t* __restrict__ out = static_cast<const uint64_t*>(out_v);
        uint64_t* o_tile = reinterpret_cast<uint64_t*>(smem + G::OUT_OFF);
#pragma unroll
        for (int q = 0; q < C::TW * C::TH / tile::THREADS; ++q) {
            const int idx = threadIdx.x + q * tile::THREADS;
            const int r = idx / C::TW, cc = idx % C::TW;
            const int64_t oi = i0 + r, oj = j0 + cc;
            const bool ok = static_cast<uint64_t>(oi) < static_cast<uint64_t>(nr) && oj < n;
            cp_async<8>(o_tile + idx, ok ? out + oi * n + oj : out, ok ? 8 : 0);
        }
    }
    cp_async_wait_all();
    __syncthreads();
}

// blockIdx = (tile column, tile row counted from row0). The evaluation stores 16-byte vectors only
// on the rows whose words start on a 16-byte boundary (vec_ok false: checked row by row), the other
// rows one element at a time. The arrays hold nr rows of the n x n grid from grid row goff; rows
// from row_end on are read as halo but not stored.
// The stencils that take the table route stage `in` and `out` with asynchronous copies and update
// `out` in the shared-memory out tile (n=16383, FP64, one application: star R=3 1620 GFLOP/s against
// 1472 with `in` staged by plain loads and `out` read by the table route itself, grid R=2 2246
// against 2155). The others, bound by HBM, stage `in` with plain loads and read `out` in the
// evaluation (star R=2: 3427 against 2909 with asynchronous copies, whose 8-byte form goes through
// L1).
template <int P, int R, int DT, int STEPS>
__global__ void __launch_bounds__(tile::THREADS, plain_min_blocks<P, R, DT, STEPS>())
    k_stencil_plain(const void* __restrict__ in, void* __restrict__ in_next, void* __restrict__ out, const int64_t n,
                    const int depth, const int64_t row0, const int64_t nr, const int64_t goff, const int64_t row_end)
{
    using C = tile::Cfg<DT>;
    using S = Smem<P, DT, R>;
    extern __shared__ __align__(128) unsigned char smem[];
    int* s_red = reinterpret_cast<int*>(smem + S::RED_OFF);
    const int64_t i0 = row0 + static_cast<int64_t>(blockIdx.y) * C::TH;
    const int64_t j0 = static_cast<int64_t>(blockIdx.x) * C::TW;
    const bool has_out = tile::tile_has_out(i0 + goff, j0, n, R, C::TW, C::TH);
    if constexpr (S::TBL) {
        stage_async<R, DT>(smem, in, out, n, nr, i0, j0, has_out);
        tile::process_tile<P, R, DT, STEPS, tile::OUT_SMEM>(smem, s_red, i0, j0, n, has_out, in_next, out, false,
                                                            depth, goff, row_end, smem + S::TBL_OFF);
    } else {
        batch::stage_tile<R, DT>(smem, in, n, nr, i0, j0);
        tile::process_tile<P, R, DT, STEPS, tile::OUT_HBM_AHEAD>(smem, s_red, i0, j0, n, has_out, in_next, out,
                                                                 false, depth, goff, row_end, nullptr);
    }
}

// The arguments of one launch: `depth` applications from in into in_next, accumulating into out,
// over the tiles of array rows [row0, row0 + rows) (rows = 0: to the last row). The arrays hold
// nr rows (0: n) of the n x n grid, from grid row goff.
struct Args {
    const void* in;
    void* in_next;
    void* out;
    int64_t n;
    int depth;
    cudaStream_t stream;
    int64_t row0;
    int64_t rows;
    int64_t nr;
    int64_t goff;
};

template <int P, int R, int DT, int STEPS>
cudaError_t launch(const Args& a)
{
    using C = tile::Cfg<DT>;
    constexpr int SM = Smem<P, DT, R>::BYTES;
    if (cudaError_t e = cudaFuncSetAttribute(k_stencil_plain<P, R, DT, STEPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM))
        return e;
    const int64_t nr = a.nr > 0 ? a.nr : a.n;
    if (a.row0 < 0 || a.row0 >= nr || a.rows < 0 || a.depth < 1 || a.goff < 0 || a.goff + nr > a.n)
        return cudaErrorInvalidValue;
    const int64_t rows = a.rows > 0 && a.rows < nr - a.row0 ? a.rows : nr - a.row0;
    const int64_t tx = (a.n + C::TW - 1) / C::TW, ty = (rows + C::TH - 1) / C::TH;
    if (ty > 65535) return cudaErrorInvalidValue;
    const dim3 grid(static_cast<unsigned>(tx), static_cast<unsigned>(ty));
    k_stencil_plain<P, R, DT, STEPS><<<grid, tile::THREADS, SM, a.stream>>>(a.in, a.in_next, a.out, a.n, a.depth, a.row0,
                                                                          nr, a.goff, a.row0 + rows);
    return cudaGetLastError();
}

// One application (depth 1: the STEPS = 1 kernel) or `depth` applications in one launch (STEPS = 0).
template <int DT>
cudaError_t launch_form(int pattern, int R, const Args& a)
{
#define PRK_PLAIN(PP, RR) \
    case RR: return a.depth == 1 ? launch<PP, RR, DT, 1>(a) : launch<PP, RR, DT, 0>(a);
    if (pattern == STAR) {
        switch (R) { PRK_PLAIN(STAR, 1) PRK_PLAIN(STAR, 2) PRK_PLAIN(STAR, 3) PRK_PLAIN(STAR, 4) PRK_PLAIN(STAR, 5) }
    } else {
        switch (R) { PRK_PLAIN(GRID, 1) PRK_PLAIN(GRID, 2) PRK_PLAIN(GRID, 3) PRK_PLAIN(GRID, 4) PRK_PLAIN(GRID, 5) }
    }
#undef PRK_PLAIN
    return cudaErrorInvalidValue;
}

// Per-form entry points (tile_plain_fp64.cu, tile_plain_fp32c.cu).
cudaError_t launch_fp64(int pattern, int R, const Args& a);
cudaError_t launch_fp32c(int pattern, int R, const Args& a);

}  // namespace plain
}  // namespace prk
