// The batched kernel for fp64 storage, family of the grid stencil of radius 4 alone (its weights are
// not powers of two: the table route), every temporal depth.
#include "batch_kernel.cuh"

namespace prk {
namespace batch {

cudaError_t launch_fp64_grid4(int steps, const Launch& L) { return launch_depth<FP64, fam_one(GRID, 4)>(steps, L); }

int ctas_per_sm_fp64_grid4(int steps) { return ctas_per_sm_depth<FP64, fam_one(GRID, 4)>(steps); }

}  // namespace batch
}  // namespace prk
