// The batched kernel for fp32c storage, family of the star stencils (radius 1 to 5), every temporal
// depth.
#include "batch_kernel.cuh"

namespace prk {
namespace batch {

cudaError_t launch_fp32c_star(int steps, const Launch& L) { return launch_depth<FP32C, FAM_F32_STAR>(steps, L); }

int ctas_per_sm_fp32c_star(int steps) { return ctas_per_sm_depth<FP32C, FAM_F32_STAR>(steps); }

}  // namespace batch
}  // namespace prk
