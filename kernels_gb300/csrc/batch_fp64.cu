// Instantiations of the batched kernel for fp64 storage, temporal depths 1, 2, 4, 8 and run-time depth.
#include "batch_kernel.cuh"

namespace prk {
namespace batch {

cudaError_t launch_fp64(int steps, const Launch& L) { return launch_depth<FP64>(steps, L); }

int ctas_per_sm_fp64(int steps)
{
    int b = 0;
    cudaError_t e = cudaErrorInvalidValue;
    switch (steps) {
    case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch<FP64, 1>, tile::THREADS, Layout<FP64>::SMEM); break;
    case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch<FP64, 2>, tile::THREADS, Layout<FP64>::SMEM); break;
    case 4: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch<FP64, 4>, tile::THREADS, Layout<FP64>::SMEM); break;
    case 8: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch<FP64, 8>, tile::THREADS, Layout<FP64>::SMEM); break;
    case 0: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch<FP64, 0>, tile::THREADS, Layout<FP64>::SMEM); break;
    }
    return e == cudaSuccess ? b : 0;
}

}  // namespace batch
}  // namespace prk
