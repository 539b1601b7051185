// The tile kernel for shapes a tensor map cannot describe: n not a multiple of the vector width
// (rows not 16-byte multiples) or buffers that are not 16-byte aligned.
//
// One CTA per tile, as in the TMA kernel, so that several tiles per SM are in flight at once. The
// `in` tile and its halo are staged in shared memory with coalesced plain loads (zero outside the
// grid), `out` is read from HBM in the evaluation, and the tile is then evaluated by the same code
// as the TMA and batched kernels (stencil_tile.cuh): the same exact routes, the same certification.
// STEPS = 1 is one application per launch; STEPS = 0 takes the number of applications at run time
// (any temporal depth, or a whole run).
#pragma once

#include "batch_kernel.cuh"

namespace prk {
namespace plain {

template <int DT, int R>
struct Smem {
    using G = tile::Geo<DT, R>;
    static constexpr int RED_OFF = (G::IN_BYTES + 127) / 128 * 128;
    static constexpr int BYTES = RED_OFF + tile::WARPS * 8;
};

// g.in[0] is `in`, g.in[1] is in_next; blockIdx = (tile column, tile row).
template <int P, int R, int DT, int STEPS>
__global__ void __launch_bounds__(tile::THREADS, tile::min_blocks<P, R, DT, STEPS, tile::TH_DEFAULT>())
    k_stencil_plain(const batch::GridDesc g, const int depth)
{
    extern __shared__ __align__(128) unsigned char smem[];
    int* s_red = reinterpret_cast<int*>(smem + Smem<DT, R>::RED_OFF);
    const int64_t t = static_cast<int64_t>(blockIdx.y) * g.tiles_x + blockIdx.x;
    batch::item<P, R, DT, STEPS>(smem, s_red, g, t, 0, depth);
}

template <int P, int R, int DT, int STEPS>
cudaError_t launch(const batch::GridDesc& g, int depth, cudaStream_t s)
{
    using C = tile::Cfg<DT>;
    constexpr int SM = Smem<DT, R>::BYTES;
    if (cudaError_t e = cudaFuncSetAttribute(k_stencil_plain<P, R, DT, STEPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM))
        return e;
    const int64_t ty = (g.n + C::TH - 1) / C::TH;
    if (ty > 65535 || (STEPS == 0 && depth < 1)) return cudaErrorInvalidValue;
    const dim3 grid(static_cast<unsigned>(g.tiles_x), static_cast<unsigned>(ty));
    k_stencil_plain<P, R, DT, STEPS><<<grid, tile::THREADS, SM, s>>>(g, depth);
    return cudaGetLastError();
}

// One application (steps = 1) or `depth` applications in one launch (steps = 0).
template <int DT>
cudaError_t launch_form(int pattern, int R, int steps, const batch::GridDesc& g, int depth, cudaStream_t s)
{
#define PRK_PLAIN(PP, RR)                                                                    \
    case RR:                                                                                 \
        return steps == 1 ? launch<PP, RR, DT, 1>(g, 1, s) : launch<PP, RR, DT, 0>(g, depth, s);
    if (steps != 0 && steps != 1) return cudaErrorInvalidValue;
    if (pattern == STAR) {
        switch (R) { PRK_PLAIN(STAR, 1) PRK_PLAIN(STAR, 2) PRK_PLAIN(STAR, 3) PRK_PLAIN(STAR, 4) PRK_PLAIN(STAR, 5) }
    } else {
        switch (R) { PRK_PLAIN(GRID, 1) PRK_PLAIN(GRID, 2) PRK_PLAIN(GRID, 3) PRK_PLAIN(GRID, 4) PRK_PLAIN(GRID, 5) }
    }
#undef PRK_PLAIN
    return cudaErrorInvalidValue;
}

// Per-form entry points (tile_plain_fp64.cu, tile_plain_fp32c.cu).
cudaError_t launch_fp64(int pattern, int R, int steps, const batch::GridDesc& g, int depth, cudaStream_t s);
cudaError_t launch_fp32c(int pattern, int R, int steps, const batch::GridDesc& g, int depth, cudaStream_t s);

}  // namespace plain
}  // namespace prk
