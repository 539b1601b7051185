// Instantiations of the TMA tile kernel for fp32c storage, star pattern, R=1..5, depths 1, 2, 4, 8, tile
// height 64 (the tall-tile variant: 8 rows per thread).
#include "stencil_tile.cuh"

namespace prk {
namespace tile {

cudaError_t launch_fp32c_star_tall(int R, int steps, const Launch& L) { return launch_pattern<STAR, FP32C, TH_TALL>(R, steps, L); }

}  // namespace tile
}  // namespace prk
