// The batched kernel for fp64 storage at temporal depth 2.
#include "batch_kernel.cuh"

namespace prk {
namespace batch {

PRK_BATCH_INSTANTIATE(FP64, 2)

}  // namespace batch
}  // namespace prk
