// The batched kernel for fp32c storage, family of the grid stencils (radius 1 to 5), every temporal
// depth.
#include "batch_kernel.cuh"

namespace prk {
namespace batch {

cudaError_t launch_fp32c_grid(int steps, const Launch& L) { return launch_depth<FP32C, FAM_F32_GRID>(steps, L); }

int ctas_per_sm_fp32c_grid(int steps) { return ctas_per_sm_depth<FP32C, FAM_F32_GRID>(steps); }

}  // namespace batch
}  // namespace prk
