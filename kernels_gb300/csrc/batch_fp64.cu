// The batched kernel for fp64 storage: the dispatch over temporal depths, and the depth-1
// instantiation. Depths 2, 4, 8 and the run-time depth are instantiated in batch_fp64_d2.cu,
// batch_fp64_d4.cu, batch_fp64_d8.cu and batch_fp64_whole.cu.
#include "batch_kernel.cuh"

namespace prk {
namespace batch {

PRK_BATCH_INSTANTIATE(FP64, 1)
PRK_BATCH_EXTERN(FP64, 2)
PRK_BATCH_EXTERN(FP64, 4)
PRK_BATCH_EXTERN(FP64, 8)
PRK_BATCH_EXTERN(FP64, 0)

cudaError_t launch_fp64(int steps, const Launch& L) { return launch_depth<FP64>(steps, L); }

int ctas_per_sm_fp64(int steps) { return ctas_per_sm_depth<FP64>(steps); }

}  // namespace batch
}  // namespace prk
