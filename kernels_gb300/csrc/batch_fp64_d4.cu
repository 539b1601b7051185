// The batched kernel for fp64 storage at temporal depth 4.
#include "batch_kernel.cuh"

namespace prk {
namespace batch {

PRK_BATCH_INSTANTIATE(FP64, 4)

}  // namespace batch
}  // namespace prk
