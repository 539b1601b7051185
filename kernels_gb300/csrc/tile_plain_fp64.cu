// Instantiations of the plain-staging tile kernel for fp64 storage: star and grid, R=1..5, one
// application per launch and run-time depth.
#include "tile_plain.cuh"

namespace prk {
namespace plain {

cudaError_t launch_fp64(int pattern, int R, const Args& a) { return launch_form<FP64>(pattern, R, a); }

}  // namespace plain
}  // namespace prk
