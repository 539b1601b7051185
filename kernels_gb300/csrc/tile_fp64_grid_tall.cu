// Instantiations of the TMA tile kernel for fp64 storage, grid pattern, R=1..5, depths 1, 2, 4, 8, tile
// height 64 (the tall-tile variant: 8 rows per thread).
#include "stencil_tile.cuh"

namespace prk {
namespace tile {

cudaError_t launch_fp64_grid_tall(int R, int steps, const Launch& L) { return launch_pattern<GRID, FP64, TH_TALL>(R, steps, L); }

}  // namespace tile
}  // namespace prk
