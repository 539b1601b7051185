// Instantiations of the TMA tile kernel for fp32c storage, star pattern, R=1..5, depths 1, 2, 4, 8, tile
// height 32 (one translation unit per storage form, pattern and tile height, so the build compiles
// them in parallel).
#include "stencil_tile.cuh"

namespace prk {
namespace tile {

cudaError_t launch_fp32c_star(int R, int steps, const Launch& L) { return launch_pattern<STAR, FP32C, TH_DEFAULT>(R, steps, L); }

}  // namespace tile
}  // namespace prk
