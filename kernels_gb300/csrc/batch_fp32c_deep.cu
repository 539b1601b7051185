// The batched kernel for fp32c storage at temporal depth 8 and at the run-time depth (whole runs).
#include "batch_kernel.cuh"

namespace prk {
namespace batch {

PRK_BATCH_INSTANTIATE(FP32C, 8)
PRK_BATCH_INSTANTIATE(FP32C, 0)

}  // namespace batch
}  // namespace prk
