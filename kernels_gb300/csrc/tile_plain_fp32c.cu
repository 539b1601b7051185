// Instantiations of the plain-staging tile kernel for FP32C storage (FP32 with compensated
// accumulation): star and grid, R=1..5, one application per launch and run-time depth.
#include "tile_plain.cuh"

namespace prk {
namespace plain {

cudaError_t launch_fp32c(int pattern, int R, const Args& a) { return launch_form<FP32C>(pattern, R, a); }

}  // namespace plain
}  // namespace prk
