// The tile kernel for shapes a tensor map cannot describe: n not a multiple of the vector width
// (rows not 16-byte multiples) or buffers that are not 16-byte aligned.
//
// One CTA per tile, as in the TMA kernel, so that several tiles per SM are in flight at once. The
// `in` tile and its halo are staged in shared memory with coalesced plain loads (zero outside the
// grid), `out` is read from HBM by the evaluation (tile::OUT_HBM_AHEAD), and the tile is evaluated
// by the same code as the TMA and batched kernels (stencil_tile.cuh): the same exact routes, the
// same certification.
// STEPS = 1 is one application per launch; STEPS = 0 takes the number of applications at run time
// (any temporal depth, or a whole run).
#pragma once

#include "batch_kernel.cuh"

namespace prk {
namespace plain {

// Shared memory: the staged `in` tile, the certification's reduction words, and for the stencils that
// take the table route (tile::table_tile) its product tables followed by its out area.
template <int P, int DT, int R>
struct Smem {
    using G = tile::Geo<DT, R>;
    static constexpr int RED_OFF = (G::IN_BYTES + 127) / 128 * 128;
    static constexpr int TBL_OFF = (RED_OFF + tile::WARPS * 8 + 15) / 16 * 16;
    static constexpr int BYTES =
        TBL_OFF + tile::table_bytes<P, R, DT>() + (tile::table_route<P, R, DT>() ? tile::table_out_bytes() : 0);
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

// blockIdx = (tile column, tile row counted from row0). The evaluation is compiled for one-by-one
// stores only (the shapes here never allow the 16-byte vectors). The arrays hold nr rows of the
// n x n grid from grid row goff; rows from row_end on are read as halo but not stored.
template <int P, int R, int DT, int STEPS>
__global__ void __launch_bounds__(tile::THREADS, plain_min_blocks<P, R, DT, STEPS>())
    k_stencil_plain(const void* __restrict__ in, void* __restrict__ in_next, void* __restrict__ out, const int64_t n,
                    const int depth, const int64_t row0, const int64_t nr, const int64_t goff, const int64_t row_end)
{
    using C = tile::Cfg<DT>;
    extern __shared__ __align__(128) unsigned char smem[];
    int* s_red = reinterpret_cast<int*>(smem + Smem<P, DT, R>::RED_OFF);
    const int64_t i0 = row0 + static_cast<int64_t>(blockIdx.y) * C::TH;
    const int64_t j0 = static_cast<int64_t>(blockIdx.x) * C::TW;
    const bool has_out = tile::tile_has_out(i0 + goff, j0, n, R, C::TW, C::TH);
    batch::stage_tile<R, DT>(smem, in, n, nr, i0, j0);
    tile::process_tile<P, R, DT, STEPS, tile::OUT_HBM_AHEAD>(
        smem, s_red, i0, j0, n, has_out, in_next, out, false, depth, goff, row_end,
        tile::table_route<P, R, DT>() ? smem + Smem<P, DT, R>::TBL_OFF : nullptr);
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
