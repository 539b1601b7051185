// prk_gb300_norm_noalloc: the interior L1 norm without any allocation.
//
// prk_gb300_norm keeps its partial sums in a device buffer that the library allocates with
// cudaMalloc on first use. Some callers cannot let a library do that: a framework whose caching
// allocator owns all device memory and budgets it, a service with a fixed memory budget, or a
// latency-critical loop where cudaMalloc's implicit device synchronisation is not acceptable. This
// entry point serves them: its scratch is a fixed-size array in the library's own device image,
// reserved when the library's module is loaded on a device and held until the process exits, and
// the caller supplies the output location as device memory.
//
// The scratch is the file-scope array below. Host code must not pass the array's name to a kernel:
// on the host that name denotes a host-side shadow, not device memory. A kernel handed it would
// fault, or, on a system where the GPU can reach host memory, silently read and write the wrong
// memory. The device address is looked up with cudaGetSymbolAddress, with the device current, on
// the first call made on that device, and kept together with the identity of the CUDA context it
// belongs to (cuCtxGetId). A later call in another context on that device (after cudaDeviceReset,
// which loads the library's module again, possibly at another address) looks it up again. The first
// call on a device, and the first after a reset, should therefore come before any stream capture.
// Every call shares the array: it is not cleared between calls (the norm kernels write every partial
// they later read, so nothing needs to start at zero), and calls that overlap on the GPU (for
// instance on two streams) race on it and give undefined results.
#include <cudaTypedefs.h>

#include <cstdio>
#include <mutex>

#include "../../include/prk_gb300.h"
#include "prk_internal.cuh"

namespace prk {

// Unique id of the calling thread's current CUDA context, 0 when there is none or the driver gives
// none. The driver entry points come through the runtime, so the library does not link libcuda.
unsigned long long current_context_id()
{
    static std::once_flag once;
    static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

}  // namespace prk

namespace {

// One partial sum per reduction block: PRK_NOALLOC_NORM_PARTIALS doubles, 8 KiB per device.
constexpr int NOALLOC_SCRATCH_DOUBLES = PRK_NOALLOC_NORM_PARTIALS;
static_assert(PRK_NOALLOC_NORM_PARTIALS == prk::NORM_BLOCKS, "the no-alloc scratch must hold every norm partial");

static __device__ __align__(256) double g_norm_scratch[NOALLOC_SCRATCH_DOUBLES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
struct ScratchAddress {
    double* ptr = nullptr;
    unsigned long long context = 0;  // cuCtxGetId of the context the address belongs to
};
ScratchAddress g_scratch_dev[MAX_DEVICES];

int fail(int code, const char* msg) { return prk::record_error(code, msg); }

// Device address of the scratch in the current device's current context: looked up once per device
// and context.
int scratch_address(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(static_cast<int>(e), "prk_gb300_norm_noalloc: cudaGetDevice failed");
    if (dev < 0 || dev >= MAX_DEVICES) return fail(PRK_ERR_LIMIT, "prk_gb300_norm_noalloc: device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_mu);
    ScratchAddress& a = g_scratch_dev[dev];
    const unsigned long long ctx = prk::current_context_id();
    if (!a.ptr || ctx == 0 || ctx != a.context) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_norm_scratch);  // also makes the device's primary context current
        if (e != cudaSuccess) {
            char msg[256];
            std::snprintf(msg, sizeof msg, "prk_gb300_norm_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return fail(static_cast<int>(e), msg);
        }
        a.ptr = static_cast<double*>(p);
        a.context = prk::current_context_id();
    }
    *out = a.ptr;
    return PRK_OK;
}

}  // namespace

extern "C" int prk_gb300_norm_noalloc(int radius, int64_t n, int dtype, const void* out, double* norm_dev, void* stream)
{
    if (dtype != PRK_FP64 && dtype != PRK_FP32C) return fail(PRK_ERR_ARG, "prk_gb300_norm_noalloc: dtype is not PRK_FP64 or PRK_FP32C");
    if (n < 1) return fail(PRK_ERR_ARG, "prk_gb300_norm_noalloc: grid dimension must be positive");
    if (n > prk::NMAX) return fail(PRK_ERR_LIMIT, "prk_gb300_norm_noalloc: grid dimension above the maximum");
    if (radius < 1 || radius > prk::RMAX || 2 * static_cast<int64_t>(radius) + 1 > n)
        return fail(PRK_ERR_ARG, "prk_gb300_norm_noalloc: stencil radius negative or too large");
    if (!out || !norm_dev) return fail(PRK_ERR_ARG, "prk_gb300_norm_noalloc: out and norm_dev must be non-null device pointers");
    // The reduction uses one partial per block, min(n-2R, NORM_BLOCKS) blocks; reject anything the
    // fixed scratch could not hold.
    const int64_t rows = n - 2 * radius;
    const int64_t partials = rows < prk::NORM_BLOCKS ? rows : prk::NORM_BLOCKS;
    if (partials > PRK_NOALLOC_NORM_PARTIALS)
        return fail(PRK_ERR_LIMIT, "prk_gb300_norm_noalloc: reduction needs more partial sums than the fixed scratch holds");
    double* scratch = nullptr;
    if (int rc = scratch_address(&scratch)) return rc;
    cudaError_t e = prk::launch_norm(radius, n, dtype, out, scratch, norm_dev, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        char msg[256];
        std::snprintf(msg, sizeof msg, "prk_gb300_norm_noalloc: launch failed: %s", cudaGetErrorString(e));
        return fail(static_cast<int>(e), msg);
    }
    return PRK_OK;
}
