// The batched kernel for fp64 storage at the run-time depth (whole runs).
#include "batch_kernel.cuh"

namespace prk {
namespace batch {

PRK_BATCH_INSTANTIATE(FP64, 0)

}  // namespace batch
}  // namespace prk
