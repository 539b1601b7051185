// The batched kernel for fp32c storage at temporal depth 8 and at the run-time depth (whole runs).
#include "batch_kernel.cuh"

namespace prk {
namespace batch {

PRK_BATCH_INSTANTIATE(FP32C, 8, FAM_ALL)
PRK_BATCH_INSTANTIATE(FP32C, 0, FAM_ALL)

}  // namespace batch
}  // namespace prk
