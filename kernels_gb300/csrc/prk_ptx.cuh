// Inline-PTX wrappers for the data movers the stencil kernels use: mbarriers and TMA
// (cp.async.bulk.tensor) tile loads into shared memory, and per-thread asynchronous copies
// (cp.async). Every wait is bounded: after the limit it
// reports failure to the caller instead of spinning forever.
#pragma once

#include <cstdint>
#include <cuda.h>

namespace prk {

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Make the initialised barrier visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Spin on the barrier phase with an iteration limit. Each try_wait suspends the thread for a
// hardware-defined interval, so the limit corresponds to seconds, far beyond any TMA completion.
constexpr uint32_t MBAR_SPIN_LIMIT = 1u << 24;

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit = MBAR_SPIN_LIMIT)
{
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 2D tiled TMA load: box at (x, y) (x the innermost coordinate, in elements) into smem dst,
// completing on `bar` with its byte count. x * element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int32_t x, int32_t y, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// Asynchronous copy (cp.async) of E bytes (4, 8 or 16) from global src to shared dst, both aligned
// to E; src_bytes = 0 writes E zero bytes without reading src. Completes with cp_async_wait_all.
template <int E>
__device__ __forceinline__ void cp_async(void* dst, const void* src, uint32_t src_bytes)
{
    static_assert(E == 4 || E == 8 || E == 16, "cp.async sizes");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(smem_addr(dst)), "l"(src), "n"(E), "r"(src_bytes)
                 : "memory");
}

// Wait for every cp.async this thread issued.
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

}  // namespace prk
