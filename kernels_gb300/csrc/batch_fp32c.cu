// The batched kernel for fp32c storage: the dispatch over temporal depths, and the instantiations
// for depths 1, 2 and 4. Depth 8 and the run-time depth are in batch_fp32c_deep.cu.
#include "batch_kernel.cuh"

namespace prk {
namespace batch {

PRK_BATCH_INSTANTIATE(FP32C, 1, FAM_ALL)
PRK_BATCH_INSTANTIATE(FP32C, 2, FAM_ALL)
PRK_BATCH_INSTANTIATE(FP32C, 4, FAM_ALL)
PRK_BATCH_EXTERN(FP32C, 8, FAM_ALL)
PRK_BATCH_EXTERN(FP32C, 0, FAM_ALL)

cudaError_t launch_fp32c(int steps, const Launch& L) { return launch_depth<FP32C, FAM_ALL>(steps, L); }

int ctas_per_sm_fp32c(int steps) { return ctas_per_sm_depth<FP32C, FAM_ALL>(steps); }

}  // namespace batch
}  // namespace prk
