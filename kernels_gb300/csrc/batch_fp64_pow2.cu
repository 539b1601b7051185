// The batched kernel for fp64 storage, family of the power-of-two stencils (star R=1,2, grid R=1),
// every temporal depth; and the host-side dispatch over all batched families.
#include "batch_kernel.cuh"

namespace prk {
namespace batch {

cudaError_t launch_fp64_pow2(int steps, const Launch& L) { return launch_depth<FP64, FAM_POW2>(steps, L); }

int ctas_per_sm_fp64_pow2(int steps) { return ctas_per_sm_depth<FP64, FAM_POW2>(steps); }

cudaError_t launch_family(int dtype, int fam, int steps, const Launch& L)
{
    if (dtype == FP32C)
        return fam == FAM_F32_STAR ? launch_fp32c_star(steps, L)
                                   : (fam == FAM_F32_GRID ? launch_fp32c_grid(steps, L) : cudaErrorInvalidValue);
    switch (fam) {
    case FAM_POW2: return launch_fp64_pow2(steps, L);
    case fam_one(STAR, 3): return launch_fp64_star3(steps, L);
    case fam_one(STAR, 4): return launch_fp64_star4(steps, L);
    case fam_one(STAR, 5): return launch_fp64_star5(steps, L);
    case fam_one(GRID, 2): return launch_fp64_grid2(steps, L);
    case fam_one(GRID, 3): return launch_fp64_grid3(steps, L);
    case fam_one(GRID, 4): return launch_fp64_grid4(steps, L);
    case fam_one(GRID, 5): return launch_fp64_grid5(steps, L);
    }
    return cudaErrorInvalidValue;
}

int ctas_per_sm_family(int dtype, int fam, int steps)
{
    if (dtype == FP32C)
        return fam == FAM_F32_STAR ? ctas_per_sm_fp32c_star(steps) : (fam == FAM_F32_GRID ? ctas_per_sm_fp32c_grid(steps) : 0);
    switch (fam) {
    case FAM_POW2: return ctas_per_sm_fp64_pow2(steps);
    case fam_one(STAR, 3): return ctas_per_sm_fp64_star3(steps);
    case fam_one(STAR, 4): return ctas_per_sm_fp64_star4(steps);
    case fam_one(STAR, 5): return ctas_per_sm_fp64_star5(steps);
    case fam_one(GRID, 2): return ctas_per_sm_fp64_grid2(steps);
    case fam_one(GRID, 3): return ctas_per_sm_fp64_grid3(steps);
    case fam_one(GRID, 4): return ctas_per_sm_fp64_grid4(steps);
    case fam_one(GRID, 5): return ctas_per_sm_fp64_grid5(steps);
    }
    return 0;
}

}  // namespace batch
}  // namespace prk
