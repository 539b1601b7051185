// C ABI of libprk_gb300.so (declared in include/prk_gb300.h): argument checks, dispatch to the
// kernel launchers, the timed iteration loop and the host-buffer entry point. Errors are returned,
// never raised: a negative PRK_ERR_* for a rejected call, a positive cudaError_t otherwise.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/prk_gb300.h"
#include "prk_internal.cuh"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
    return fail(static_cast<int>(e), "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

#define PRK_CUDA(call, what)                              \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

int check_common(int radius, int64_t n, int dtype)
{
    if (dtype != PRK_FP64 && dtype != PRK_FP32C) return fail(PRK_ERR_ARG, "dtype %d is not PRK_FP64 or PRK_FP32C", dtype);
    if (n < 1) return fail(PRK_ERR_ARG, "grid dimension must be positive (n=%lld)", static_cast<long long>(n));
    if (n > prk::NMAX) return fail(PRK_ERR_LIMIT, "grid dimension %lld above the maximum %lld", static_cast<long long>(n),
                                   static_cast<long long>(prk::NMAX));
    if (radius < 1 || radius > prk::RMAX || 2 * static_cast<int64_t>(radius) + 1 > n)
        return fail(PRK_ERR_ARG, "stencil radius %d negative or too large for n=%lld (1 <= R <= 5, 2R+1 <= n)", radius,
                    static_cast<long long>(n));
    return PRK_OK;
}

int check_stencil(int pattern, int radius, int64_t n, int dtype)
{
    if (pattern != PRK_STAR && pattern != PRK_GRID) return fail(PRK_ERR_ARG, "pattern %d is not PRK_STAR or PRK_GRID", pattern);
    return check_common(radius, n, dtype);
}

bool overlaps(const void* a, int64_t abytes, const void* b, int64_t bbytes)
{
    const char* pa = static_cast<const char*>(a);
    const char* pb = static_cast<const char*>(b);
    return pa < pb + bbytes && pb < pa + abytes;
}

// Library-owned device scratch: NORM_BLOCKS partial sums and the result for the norm, and the
// status word the tile kernels set when a bounded wait gives up. One allocation per device, kept
// until the process exits, with the id of the context it was made in: in a new context on the device
// (after cudaDeviceReset, which freed it) it is allocated again.
struct DevScratch {
    double* norm = nullptr;
    unsigned* status = nullptr;
    unsigned long long context = 0;
};
std::mutex g_scratch_mu;
std::vector<DevScratch> g_scratch;

int dev_scratch(DevScratch* out)
{
    int dev = 0;
    PRK_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (static_cast<int>(g_scratch.size()) <= dev) g_scratch.resize(dev + 1);
    const unsigned long long ctx = prk::current_context_id();
    if (g_scratch[dev].norm && ctx != 0 && g_scratch[dev].context != 0 && ctx != g_scratch[dev].context)
        g_scratch[dev] = DevScratch{};  // the old context and its memory are gone
    if (!g_scratch[dev].norm) {
        void* p = nullptr;
        const size_t bytes = (prk::NORM_BLOCKS + 1) * sizeof(double) + 256;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(PRK_ERR_NOMEM, "cudaMalloc of the library scratch failed: %s", cudaGetErrorString(e));
        }
        e = cudaMemset(p, 0, bytes);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemset of the library scratch");
        g_scratch[dev].norm = static_cast<double*>(p);
        g_scratch[dev].status = reinterpret_cast<unsigned*>(static_cast<char*>(p) + (prk::NORM_BLOCKS + 1) * sizeof(double));
        g_scratch[dev].context = prk::current_context_id();
    }
    *out = g_scratch[dev];
    return PRK_OK;
}

int norm_scratch(double** out)
{
    DevScratch d;
    if (int rc = dev_scratch(&d)) return rc;
    *out = d.norm;
    return PRK_OK;
}

// Device buffers and streams of prk_gb300_run_host, kept between calls (the buffers grown when a
// larger grid comes) and freed by prk_gb300_release. Streams: copies in, copies out, and two for
// the band launches.
struct HostWorkspace {
    void* d[3] = {nullptr, nullptr, nullptr};
    int64_t in_bytes = 0, out_bytes = 0;
    cudaStream_t s[4] = {nullptr, nullptr, nullptr, nullptr};
    unsigned long long context = 0;  // the context the buffers and streams belong to
};
std::mutex g_host_mu;
std::vector<HostWorkspace> g_host_ws;

// Kernel selection: 0 = automatic (TMA tiles where eligible), 1 = generic only, 2 = TMA required.
// Atomic, so that prk_gb300_config may be called while other threads run stencils.
std::atomic<int> g_kernel_choice{0};
// Set for the duration of a tuned run whose tuning chose the generic kernels, or a tile height.
thread_local bool t_force_generic = false;
thread_local int t_tile_rows = 32;

int launch_one(int pattern, int radius, int64_t n, int dtype, const void* in, void* in_next, void* out, cudaStream_t s)
{
    prk::StencilCall c{pattern, radius, n, dtype, in, in_next, out, s};
    const bool tiles = g_kernel_choice != 1 && !t_force_generic;
    const bool tma = tiles && prk::tma_eligible(c);
    if (g_kernel_choice == 2 && !tma) return fail(PRK_ERR_ARG, "the TMA tile kernel was required but the call is not eligible");
    if (tma) {
        DevScratch d;
        if (int rc = dev_scratch(&d)) return rc;
        PRK_CUDA(prk::launch_stencil_tma(c, 1, d.status, t_tile_rows), "stencil launch (TMA tiles)");
    } else if (tiles && prk::plain_eligible(c)) {
        PRK_CUDA(prk::launch_stencil_plain(c, 1), "stencil launch (plain-staged tiles)");
    } else {
        PRK_CUDA(prk::launch_stencil_generic(c), "stencil launch");
    }
    return PRK_OK;
}

// `steps` fused applications from in into in_next in one launch (TMA tiles only).
int launch_steps(int pattern, int radius, int64_t n, int dtype, int steps, const void* in, void* in_next, void* out,
                 cudaStream_t s)
{
    prk::StencilCall c{pattern, radius, n, dtype, in, in_next, out, s};
    if (!prk::tma_depth_ok(steps)) return fail(PRK_ERR_ARG, "temporal depth %d is not 1, 2, 4 or 8", steps);
    if (g_kernel_choice == 1) return fail(PRK_ERR_ARG, "temporal blocking needs the tile kernels");
    if (!prk::tma_eligible(c)) {
        if (g_kernel_choice == 2 || !prk::plain_eligible(c))
            return fail(PRK_ERR_ARG, "temporal blocking needs the tile kernels: buffers aligned to their element size%s",
                        g_kernel_choice == 2 ? ", 16-byte-aligned with n a multiple of the vector width for TMA" : "");
        PRK_CUDA(prk::launch_stencil_plain(c, steps), "stencil launch (plain-staged tiles, temporal)");
        return PRK_OK;
    }
    DevScratch d;
    if (int rc = dev_scratch(&d)) return rc;
    PRK_CUDA(prk::launch_stencil_tma(c, steps, d.status, t_tile_rows), "stencil launch (TMA tiles, temporal)");
    return PRK_OK;
}

// Reads and clears the device status word (synchronises the device).
int check_status()
{
    DevScratch d;
    if (int rc = dev_scratch(&d)) return rc;
    unsigned st = 0;
    PRK_CUDA(cudaMemcpy(&st, d.status, sizeof st, cudaMemcpyDeviceToHost), "status read");
    if (st) {
        PRK_CUDA(cudaMemset(d.status, 0, sizeof st), "status clear");
        return fail(PRK_ERR_TIMEOUT, "a bounded device-side wait gave up (status 0x%x)", st);
    }
    return PRK_OK;
}

}  // namespace

int prk::record_error(int code, const char* msg) { return fail(code, "%s", msg); }

extern "C" {

const char* prk_gb300_last_error(void) { return g_last_error.c_str(); }

const char* prk_gb300_version(void) { return "prk_gb300 0.2.0 (sm_103a)"; }

int prk_gb300_config(int key, int value)
{
    if (key == PRK_CFG_KERNEL) {
        if (value < 0 || value > 2) return fail(PRK_ERR_ARG, "PRK_CFG_KERNEL takes 0 (auto), 1 (generic) or 2 (TMA)");
        return g_kernel_choice.exchange(value);
    }
    return fail(PRK_ERR_ARG, "unknown configuration key %d", key);
}

int prk_gb300_status(void) { return check_status(); }

int prk_gb300_selftest_timeout(void)
{
    if (int rc = check_status()) return rc;  // start from a clear status word
    DevScratch d;
    if (int rc = dev_scratch(&d)) return rc;
    PRK_CUDA(prk::launch_wait_selftest(d.status, nullptr), "self-test launch");
    PRK_CUDA(cudaDeviceSynchronize(), "self-test");
    return check_status();
}

int prk_gb300_probe_dadd(double* adds_per_second)
{
    if (!adds_per_second) return fail(PRK_ERR_ARG, "adds_per_second must be non-null");
    DevScratch d;
    if (int rc = dev_scratch(&d)) return rc;
    int dev = 0, sms = 0;
    PRK_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    PRK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
    const int blocks = sms * 8, iters = 4096;
    cudaStream_t s = nullptr;
    PRK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = PRK_OK;
    do {
        cudaError_t ce;
        if ((ce = cudaEventCreate(&e0)) != cudaSuccess || (ce = cudaEventCreate(&e1)) != cudaSuccess) { rc = cuda_fail(ce, "cudaEventCreate"); break; }
        if ((ce = prk::launch_dadd_probe(d.norm, blocks, iters / 16, 0.5, s)) != cudaSuccess) { rc = cuda_fail(ce, "probe launch"); break; }
        cudaEventRecord(e0, s);
        if ((ce = prk::launch_dadd_probe(d.norm, blocks, iters, 0.5, s)) != cudaSuccess) { rc = cuda_fail(ce, "probe launch"); break; }
        cudaEventRecord(e1, s);
        if ((ce = cudaEventSynchronize(e1)) != cudaSuccess) { rc = cuda_fail(ce, "probe"); break; }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        *adds_per_second = static_cast<double>(blocks) * 256.0 * 8.0 * (iters + 1) / (ms * 1e-3);
    } while (false);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return rc;
}

int prk_gb300_route_split(int pattern, int radius, int depth, int* fixed_adds, int* binary64_adds)
{
    if (!fixed_adds || !binary64_adds) return fail(PRK_ERR_ARG, "null output");
    if (pattern != PRK_STAR && pattern != PRK_GRID) return fail(PRK_ERR_ARG, "pattern %d is not PRK_STAR or PRK_GRID", pattern);
    if (radius < 1 || radius > prk::RMAX) return fail(PRK_ERR_ARG, "radius %d outside 1..5", radius);
    if (depth < 1) return fail(PRK_ERR_ARG, "depth %d is not positive", depth);
    if (prk::table_route_split(pattern, radius, depth, fixed_adds, binary64_adds) != 0)
        return fail(PRK_ERR_ARG, "the weights of this stencil are powers of two: its FP64 form takes the exact routes");
    return PRK_OK;
}

int64_t prk_gb300_bytes(int64_t n, int dtype, int role)
{
    if (n < 1 || (dtype != PRK_FP64 && dtype != PRK_FP32C)) return -1;
    return n * n * (role == 0 ? prk::in_elem_bytes(dtype) : prk::out_elem_bytes(dtype));
}

double prk_gb300_flops(int pattern, int radius, int64_t n)
{
    const double act = static_cast<double>(n - 2 * radius) * static_cast<double>(n - 2 * radius);
    return (2.0 * prk::stencil_size(pattern == PRK_GRID ? prk::GRID : prk::STAR, radius) + 1.0) * act;
}

int prk_gb300_stencil(int pattern, int radius, int64_t n, int dtype, const void* in, void* in_next, void* out, void* stream)
{
    if (int rc = check_stencil(pattern, radius, n, dtype)) return rc;
    if (!in || !out) return fail(PRK_ERR_ARG, "in and out must be non-null device pointers");
    const int64_t ib = prk_gb300_bytes(n, dtype, 0), ob = prk_gb300_bytes(n, dtype, 1);
    if (overlaps(in, ib, out, ob)) return fail(PRK_ERR_ARG, "in and out overlap");
    if (in_next && (overlaps(in_next, ib, in, ib) || overlaps(in_next, ib, out, ob)))
        return fail(PRK_ERR_ARG, "in_next overlaps in or out");
    return launch_one(pattern, radius, n, dtype, in, in_next, out, static_cast<cudaStream_t>(stream));
}

int prk_gb300_stencil_steps(int pattern, int radius, int64_t n, int dtype, int steps, const void* in, void* in_next,
                            void* out, void* stream)
{
    if (int rc = check_stencil(pattern, radius, n, dtype)) return rc;
    if (!in || !in_next || !out) return fail(PRK_ERR_ARG, "in, in_next and out must be non-null device pointers");
    const int64_t ib = prk_gb300_bytes(n, dtype, 0), ob = prk_gb300_bytes(n, dtype, 1);
    if (overlaps(in, ib, out, ob) || overlaps(in_next, ib, in, ib) || overlaps(in_next, ib, out, ob))
        return fail(PRK_ERR_ARG, "buffers overlap");
    return launch_steps(pattern, radius, n, dtype, steps, in, in_next, out, static_cast<cudaStream_t>(stream));
}

int prk_gb300_add(int64_t n, int dtype, void* in, void* stream)
{
    if (dtype != PRK_FP64 && dtype != PRK_FP32C) return fail(PRK_ERR_ARG, "dtype %d is not PRK_FP64 or PRK_FP32C", dtype);
    if (n < 1 || !in) return fail(PRK_ERR_ARG, "n must be positive and in non-null");
    PRK_CUDA(prk::launch_add(n, dtype, in, static_cast<cudaStream_t>(stream)), "add launch");
    return PRK_OK;
}

int prk_gb300_init(int64_t n, int dtype, void* in, void* out, void* stream)
{
    if (dtype != PRK_FP64 && dtype != PRK_FP32C) return fail(PRK_ERR_ARG, "dtype %d is not PRK_FP64 or PRK_FP32C", dtype);
    if (n < 1 || !in || !out) return fail(PRK_ERR_ARG, "n must be positive and in, out non-null");
    PRK_CUDA(prk::launch_init(n, dtype, in, out, static_cast<cudaStream_t>(stream)), "init launch");
    return PRK_OK;
}

int prk_gb300_norm(int radius, int64_t n, int dtype, const void* out, double* norm, void* stream)
{
    if (int rc = check_common(radius, n, dtype)) return rc;
    if (!out || !norm) return fail(PRK_ERR_ARG, "out and norm must be non-null");
    double* scratch = nullptr;
    if (int rc = norm_scratch(&scratch)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PRK_CUDA(prk::launch_norm(radius, n, dtype, out, scratch, scratch + prk::NORM_BLOCKS, s), "norm launch");
    PRK_CUDA(cudaMemcpyAsync(norm, scratch + prk::NORM_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, s), "norm copy");
    PRK_CUDA(cudaStreamSynchronize(s), "norm synchronize");
    return PRK_OK;
}

int prk_gb300_run(int pattern, int radius, int64_t n, int dtype, int iterations, void* in_a, void* in_b, void* out,
                  int flags, double* elapsed_s, int* final_in, void* stream)
{
    if (int rc = check_stencil(pattern, radius, n, dtype)) return rc;
    if (iterations < 1) return fail(PRK_ERR_ARG, "iterations must be >= 1");
    const bool unfused = (flags & PRK_RUN_UNFUSED) != 0;
    const bool graph = (flags & PRK_RUN_GRAPH) != 0;
    bool whole = (flags & PRK_RUN_WHOLE) != 0;
    if (whole && unfused) return fail(PRK_ERR_ARG, "PRK_RUN_WHOLE is a fused form");
    int depth = (flags >> 8) & 0xFF;
    if (depth == 0) depth = 1;
    if (!prk::tma_depth_ok(depth)) return fail(PRK_ERR_ARG, "temporal depth %d is not 1, 2, 4 or 8", depth);
    if (!in_a || !out || (!unfused && !in_b)) return fail(PRK_ERR_ARG, "null buffer");
    bool tuned_generic = false;
    int rows = (flags & PRK_RUN_TALL) ? 64 : 32;
    if ((flags & PRK_RUN_TUNED) && !unfused && !whole) {
        prk_gb300_tuning t{};
        if (int rc = prk_gb300_tune(pattern, radius, n, dtype, 0, &t)) return rc;
        depth = t.depth > 0 ? t.depth : 1;
        whole = t.depth == 0 && g_kernel_choice != 1;  // the generic kernels run one application per launch
        tuned_generic = t.kernel == 1;
        if (!tuned_generic) rows = t.tile_rows;
    }
    struct TuneScope {  // the tuned kernel family and tile height hold for this run only
        bool generic;
        int prev_rows;
        TuneScope(bool g, int r) : generic(g), prev_rows(t_tile_rows)
        {
            if (generic) t_force_generic = true;
            t_tile_rows = r;
        }
        ~TuneScope()
        {
            if (generic) t_force_generic = false;
            t_tile_rows = prev_rows;
        }
    } tune_scope(tuned_generic, rows);
    const int64_t ib = prk_gb300_bytes(n, dtype, 0), ob = prk_gb300_bytes(n, dtype, 1);
    if (overlaps(in_a, ib, out, ob) || (!unfused && (overlaps(in_b, ib, out, ob) || overlaps(in_a, ib, in_b, ib))))
        return fail(PRK_ERR_ARG, "buffers overlap");

    cudaStream_t user = static_cast<cudaStream_t>(stream);
    cudaStream_t s = user;
    cudaStream_t own = nullptr;
    if (graph && s == nullptr) {  // capture needs a non-legacy stream
        PRK_CUDA(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking), "cudaStreamCreate");
        s = own;
    }
    void* bufs[2] = {in_a, in_b};
    int cur = 0;
    {
        prk::StencilCall probe{pattern, radius, n, dtype, in_a, in_b, out, nullptr};
        if (unfused || g_kernel_choice == 1 || t_force_generic ||
            (!prk::tma_eligible(probe) && (g_kernel_choice == 2 || !prk::plain_eligible(probe))))
            depth = 1;
    }
    auto step = [&](cudaStream_t st) -> int {
        if (unfused) {
            if (int rc = launch_one(pattern, radius, n, dtype, in_a, nullptr, out, st)) return rc;
            PRK_CUDA(prk::launch_add(n, dtype, in_a, st), "add launch");
        } else {
            if (int rc = launch_one(pattern, radius, n, dtype, bufs[cur], bufs[cur ^ 1], out, st)) return rc;
            cur ^= 1;
        }
        return PRK_OK;
    };
    bool whole_tma = true;
    if (whole) {
        prk::StencilCall probe{pattern, radius, n, dtype, in_a, in_b, out, nullptr};
        whole_tma = prk::tma_eligible(probe);
        if (g_kernel_choice == 1 || (!whole_tma && (g_kernel_choice == 2 || !prk::plain_eligible(probe))))
            return fail(PRK_ERR_ARG, "PRK_RUN_WHOLE needs the tile kernels: buffers aligned to their element size");
    }
    // `count` applications: one launch (whole run), or launches of the temporal depth with the
    // remainder in powers of two.
    auto steps = [&](cudaStream_t st, int count) -> int {
        if (whole) {
            prk::StencilCall c{pattern, radius, n, dtype, bufs[cur], bufs[cur ^ 1], out, st};
            if (whole_tma) {
                DevScratch dsc;
                if (int rc = dev_scratch(&dsc)) return rc;
                PRK_CUDA(prk::launch_stencil_tma_band(c, count, 0, n, dsc.status), "stencil launch (TMA tiles, whole run)");
            } else {
                PRK_CUDA(prk::launch_stencil_plain(c, count), "stencil launch (plain-staged tiles, whole run)");
            }
            cur ^= 1;
            return PRK_OK;
        }
        if (depth == 1) {
            for (int i = 0; i < count; ++i)
                if (int rc = step(st)) return rc;
            return PRK_OK;
        }
        while (count > 0) {
            int d = depth;
            while (d > count) d >>= 1;
            if (int rc = launch_steps(pattern, radius, n, dtype, d, bufs[cur], bufs[cur ^ 1], out, st)) return rc;
            cur ^= 1;
            count -= d;
        }
        return PRK_OK;
    };

    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    int rc = PRK_OK;
    do {
        cudaError_t ce;
        if (own) {  // order the private stream after prior work on the legacy stream
            cudaEvent_t dep;
            if ((ce = cudaEventCreateWithFlags(&dep, cudaEventDisableTiming)) != cudaSuccess) { rc = cuda_fail(ce, "cudaEventCreate"); break; }
            cudaEventRecord(dep, nullptr);
            cudaStreamWaitEvent(s, dep, 0);
            cudaEventDestroy(dep);
        }
        if ((ce = cudaEventCreate(&e0)) != cudaSuccess || (ce = cudaEventCreate(&e1)) != cudaSuccess) { rc = cuda_fail(ce, "cudaEventCreate"); break; }
        if ((rc = step(s)) != PRK_OK) break;  // iteration 0: untimed warm-up
        if (graph) {
            if ((ce = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) { rc = cuda_fail(ce, "cudaStreamBeginCapture"); break; }
            rc = steps(s, iterations);
            cudaError_t ec = cudaStreamEndCapture(s, &g);
            if (rc != PRK_OK) break;
            if (ec != cudaSuccess) { rc = cuda_fail(ec, "cudaStreamEndCapture"); break; }
            if ((ce = cudaGraphInstantiate(&ge, g, 0)) != cudaSuccess) { rc = cuda_fail(ce, "cudaGraphInstantiate"); break; }
            if ((ce = cudaGraphUpload(ge, s)) != cudaSuccess) { rc = cuda_fail(ce, "cudaGraphUpload"); break; }
            cudaEventRecord(e0, s);
            if ((ce = cudaGraphLaunch(ge, s)) != cudaSuccess) { rc = cuda_fail(ce, "cudaGraphLaunch"); break; }
            cudaEventRecord(e1, s);
        } else {
            cudaEventRecord(e0, s);
            rc = steps(s, iterations);
            if (rc != PRK_OK) break;
            cudaEventRecord(e1, s);
        }
        if ((ce = cudaEventSynchronize(e1)) != cudaSuccess) { rc = cuda_fail(ce, "iteration loop"); break; }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (elapsed_s) *elapsed_s = ms * 1e-3;
        if (final_in) *final_in = unfused ? 0 : cur;
        rc = check_status();
    } while (false);
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (own) {
        cudaStreamSynchronize(own);
        cudaStreamDestroy(own);
    }
    return rc;
}

int prk_gb300_slab_run(int pattern, int radius, int64_t n, int dtype, int apps, int64_t row_begin, int64_t row_end,
                       const void* in, void* in_next, void* out, void* stream)
{
    if (int rc = check_stencil(pattern, radius, n, dtype)) return rc;
    if (apps < 1) return fail(PRK_ERR_ARG, "apps must be >= 1");
    if (row_begin < 0 || row_end > n || row_begin >= row_end)
        return fail(PRK_ERR_ARG, "slab rows [%lld, %lld) are empty or outside the grid of %lld rows",
                    static_cast<long long>(row_begin), static_cast<long long>(row_end), static_cast<long long>(n));
    if (!in || !in_next || !out) return fail(PRK_ERR_ARG, "in, in_next and out must be non-null device pointers");
    const int64_t halo_begin = std::max<int64_t>(0, row_begin - radius);
    const int64_t halo_end = std::min<int64_t>(n, row_end + radius);
    const int64_t nr = halo_end - halo_begin;
    const int64_t ib = nr * n * prk::in_elem_bytes(dtype), ob = nr * n * prk::out_elem_bytes(dtype);
    if (overlaps(in, ib, out, ob) || overlaps(in_next, ib, in, ib) || overlaps(in_next, ib, out, ob))
        return fail(PRK_ERR_ARG, "buffers overlap");
    if (g_kernel_choice == 1) return fail(PRK_ERR_ARG, "slab runs need the tile kernels");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    prk::StencilCall c{pattern, radius, n, dtype, in, in_next, out, s, nr, halo_begin};
    const int64_t row0 = row_begin - halo_begin, rows = row_end - row_begin;
    if (prk::tma_eligible(c)) {
        DevScratch d;
        if (int rc = dev_scratch(&d)) return rc;
        if (prk::tma_depth_ok(apps))
            PRK_CUDA(prk::launch_stencil_tma_rows(c, apps, row0, rows, d.status), "slab launch (TMA tiles)");
        else
            PRK_CUDA(prk::launch_stencil_tma_band(c, apps, row0, rows, d.status), "slab launch (TMA tiles)");
        return PRK_OK;
    }
    if (g_kernel_choice == 2 || !prk::plain_eligible(c))
        return fail(PRK_ERR_ARG, "slab buffers must be aligned to their element size%s",
                    g_kernel_choice == 2 ? ", 16-byte-aligned with n a multiple of the vector width for TMA" : "");
    PRK_CUDA(prk::launch_stencil_plain(c, apps, row0, rows), "slab launch (plain-staged tiles)");
    return PRK_OK;
}

int prk_gb300_slab_norm(int radius, int64_t n, int dtype, int64_t row_begin, int64_t row_end, const void* out,
                        double* l1_sum, void* stream)
{
    if (int rc = check_common(radius, n, dtype)) return rc;
    if (row_begin < 0 || row_end > n || row_begin >= row_end)
        return fail(PRK_ERR_ARG, "slab rows [%lld, %lld) are empty or outside the grid of %lld rows",
                    static_cast<long long>(row_begin), static_cast<long long>(row_end), static_cast<long long>(n));
    if (!out || !l1_sum) return fail(PRK_ERR_ARG, "out and l1_sum must be non-null");
    double* scratch = nullptr;
    if (int rc = norm_scratch(&scratch)) return rc;
    const int64_t halo_begin = std::max<int64_t>(0, row_begin - radius);
    const int64_t lo = std::max<int64_t>(row_begin, radius) - halo_begin;
    const int64_t hi = std::min<int64_t>(row_end, n - radius) - halo_begin;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PRK_CUDA(prk::launch_norm_rows(radius, n, dtype, out, lo, hi, 1.0, scratch, scratch + prk::NORM_BLOCKS, s),
             "slab norm launch");
    PRK_CUDA(cudaMemcpyAsync(l1_sum, scratch + prk::NORM_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, s), "norm copy");
    PRK_CUDA(cudaStreamSynchronize(s), "norm synchronize");
    return PRK_OK;
}

}  // extern "C"

namespace {

// Events of one banded run, destroyed on scope exit.
struct BandEvents {
    std::vector<cudaEvent_t> ev;
    ~BandEvents()
    {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
    cudaError_t make(size_t count, unsigned flags)
    {
        ev.assign(count, nullptr);
        for (cudaEvent_t& e : ev)
            if (cudaError_t ce = cudaEventCreateWithFlags(&e, flags)) return ce;
        return cudaSuccess;
    }
};

// The host-buffer run in bands of rows. `in` evolves pointwise, so a band's `out` after every
// application depends only on its own rows of `out` and its rows of `in` with R more on either
// side, and one launch of the run-time-depth tile kernel carries all `apps` applications of the
// band. The bands' copies to the device go in order on one stream; band b is launched once its
// rows and the next band's (its lower halo) have landed, on one of two streams so that one band's
// last wave overlaps the next band's first; its rows go back to the host as soon as it is done.
// Copies in, evaluation and copies out of different bands overlap.
int run_host_banded(HostWorkspace& ws, int pattern, int radius, int64_t n, int dtype, int apps, const void* h_in,
                    void* h_out, void* h_in_final, double* norm, double* kernel_s)
{
    DevScratch sc;
    if (int rc = dev_scratch(&sc)) return rc;
    for (cudaStream_t& st : ws.s)
        if (!st) PRK_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    cudaStream_t s_in = ws.s[0], s_out = ws.s[1], s_ev[2] = {ws.s[2], ws.s[3]};
    struct Drain {  // no copy of the caller's host buffers outlives the call, on any return
        cudaStream_t* s;
        ~Drain()
        {
            for (int i = 0; i < 4; ++i) cudaStreamSynchronize(s[i]);
        }
    } drain{ws.s};
    const int64_t es = dtype == PRK_FP64 ? 8 : 4;  // bytes per `in` element; `out` has 8
    const int64_t band = std::max<int64_t>(128, (n / 32 + 31) / 32 * 32);
    const int nb = static_cast<int>((n + band - 1) / band);
    BandEvents landed, done, span;
    PRK_CUDA(landed.make(nb, cudaEventDisableTiming), "cudaEventCreate");
    PRK_CUDA(done.make(nb, cudaEventDisableTiming), "cudaEventCreate");
    PRK_CUDA(span.make(2, cudaEventDefault), "cudaEventCreate");
    char* d_in = static_cast<char*>(ws.d[0]);
    char* d_fin = static_cast<char*>(ws.d[1]);
    char* d_out = static_cast<char*>(ws.d[2]);
    const char* hi = static_cast<const char*>(h_in);
    char* ho = static_cast<char*>(h_out);
    char* hf = static_cast<char*>(h_in_final);
    for (int b = 0; b < nb; ++b) {
        const int64_t r0 = b * band, rows = std::min(band, n - r0);
        PRK_CUDA(cudaMemcpyAsync(d_in + r0 * n * es, hi + r0 * n * es, rows * n * es, cudaMemcpyHostToDevice, s_in),
                 "host to device copy");
        PRK_CUDA(cudaMemcpyAsync(d_out + r0 * n * 8, ho + r0 * n * 8, rows * n * 8, cudaMemcpyHostToDevice, s_in),
                 "host to device copy");
        PRK_CUDA(cudaEventRecord(landed.ev[b], s_in), "cudaEventRecord");
    }
    for (int b = 0; b < nb; ++b) {
        const int64_t r0 = b * band, rows = std::min(band, n - r0);
        cudaStream_t st = s_ev[b & 1];
        PRK_CUDA(cudaStreamWaitEvent(st, landed.ev[b + 1 < nb ? b + 1 : b], 0), "cudaStreamWaitEvent");
        if (b == 0) PRK_CUDA(cudaEventRecord(span.ev[0], st), "cudaEventRecord");
        prk::StencilCall c{pattern, radius, n, dtype, d_in, d_fin, d_out, st};
        if (prk::tma_eligible(c))
            PRK_CUDA(prk::launch_stencil_tma_band(c, apps, r0, rows, sc.status), "band launch (TMA tiles)");
        else
            PRK_CUDA(prk::launch_stencil_plain(c, apps, r0, rows), "band launch (plain-staged tiles)");
        PRK_CUDA(cudaEventRecord(done.ev[b], st), "cudaEventRecord");
        PRK_CUDA(cudaStreamWaitEvent(s_out, done.ev[b], 0), "cudaStreamWaitEvent");
        PRK_CUDA(cudaMemcpyAsync(ho + r0 * n * 8, d_out + r0 * n * 8, rows * n * 8, cudaMemcpyDeviceToHost, s_out),
                 "device to host copy");
        if (hf)
            PRK_CUDA(cudaMemcpyAsync(hf + r0 * n * es, d_fin + r0 * n * es, rows * n * es, cudaMemcpyDeviceToHost, s_out),
                     "device to host copy");
    }
    // the norm after every band, on the first evaluation stream (the last two bands cover both)
    if (nb > 1) PRK_CUDA(cudaStreamWaitEvent(s_ev[0], done.ev[nb - 2], 0), "cudaStreamWaitEvent");
    PRK_CUDA(cudaStreamWaitEvent(s_ev[0], done.ev[nb - 1], 0), "cudaStreamWaitEvent");
    PRK_CUDA(cudaEventRecord(span.ev[1], s_ev[0]), "cudaEventRecord");
    if (norm) {
        if (int rc = prk_gb300_norm(radius, n, dtype, d_out, norm, s_ev[0])) return rc;
    }
    PRK_CUDA(cudaStreamSynchronize(s_out), "copies back");
    PRK_CUDA(cudaStreamSynchronize(s_ev[0]), "band evaluation");
    PRK_CUDA(cudaStreamSynchronize(s_ev[1]), "band evaluation");
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, span.ev[0], span.ev[1]);
    if (kernel_s) *kernel_s = ms * 1e-3;
    return check_status();
}

}  // namespace

extern "C" {

int prk_gb300_run_host(int pattern, int radius, int64_t n, int dtype, int iterations, const void* h_in, void* h_out,
                       void* h_in_final, double* norm, double* elapsed_s, double* kernel_s)
{
    const auto t0 = std::chrono::steady_clock::now();
    if (int rc = check_stencil(pattern, radius, n, dtype)) return rc;
    if (iterations < 1 || iterations > (1 << 30)) return fail(PRK_ERR_ARG, "iterations must be in 1..2^30");
    if (!h_in || !h_out) return fail(PRK_ERR_ARG, "h_in and h_out must be non-null");
    const int64_t ib = prk_gb300_bytes(n, dtype, 0), ob = prk_gb300_bytes(n, dtype, 1);
    int dev = 0;
    PRK_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lock(g_host_mu);  // one host-buffer run per process at a time
    if (static_cast<int>(g_host_ws.size()) <= dev) g_host_ws.resize(dev + 1);
    HostWorkspace& ws = g_host_ws[dev];
    {
        const unsigned long long ctx = prk::current_context_id();
        if (ws.context != 0 && ctx != 0 && ctx != ws.context) ws = HostWorkspace{};  // freed with the old context
    }
    int rc = PRK_OK;
    do {
        cudaError_t ce;
        if (ws.in_bytes < ib || ws.out_bytes < ob) {  // grow the cached device buffers
            for (void*& p : ws.d) {
                if (p) cudaFree(p);
                p = nullptr;
            }
            ws.in_bytes = ws.out_bytes = 0;
            if ((ce = cudaMalloc(&ws.d[0], ib)) != cudaSuccess || (ce = cudaMalloc(&ws.d[1], ib)) != cudaSuccess ||
                (ce = cudaMalloc(&ws.d[2], ob)) != cudaSuccess) {
                cudaGetLastError();
                for (void*& p : ws.d) {
                    if (p) cudaFree(p);
                    p = nullptr;
                }
                rc = fail(PRK_ERR_NOMEM, "device allocation of %lld bytes failed: %s", static_cast<long long>(2 * ib + ob),
                          cudaGetErrorString(ce));
                break;
            }
            ws.in_bytes = ib;
            ws.out_bytes = ob;
            ws.context = prk::current_context_id();
        }
        void** d = ws.d;
        {
            prk::StencilCall probe{pattern, radius, n, dtype, d[0], d[1], d[2], nullptr};
            const bool tiles = prk::tma_eligible(probe) || (g_kernel_choice == 0 && prk::plain_eligible(probe));
            if (g_kernel_choice != 1 && tiles) {  // iteration 0 plus `iterations`
                rc = run_host_banded(ws, pattern, radius, n, dtype, iterations + 1, h_in, h_out, h_in_final, norm, kernel_s);
                break;
            }
        }
        if ((ce = cudaMemcpy(d[0], h_in, ib, cudaMemcpyHostToDevice)) != cudaSuccess ||
            (ce = cudaMemcpy(d[2], h_out, ob, cudaMemcpyHostToDevice)) != cudaSuccess) { rc = cuda_fail(ce, "host to device copy"); break; }
        int fin = 0;
        double ks = 0.0;
        if ((rc = prk_gb300_run(pattern, radius, n, dtype, iterations, d[0], d[1], d[2], PRK_RUN_TUNED, &ks, &fin, nullptr)) != PRK_OK) break;
        if ((ce = cudaMemcpy(h_out, d[2], ob, cudaMemcpyDeviceToHost)) != cudaSuccess) { rc = cuda_fail(ce, "device to host copy"); break; }
        if (h_in_final && (ce = cudaMemcpy(h_in_final, d[fin], ib, cudaMemcpyDeviceToHost)) != cudaSuccess) { rc = cuda_fail(ce, "device to host copy"); break; }
        if (norm && (rc = prk_gb300_norm(radius, n, dtype, d[2], norm, nullptr)) != PRK_OK) break;
        if (kernel_s) *kernel_s = ks;
    } while (false);
    if (elapsed_s) *elapsed_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

int prk_gb300_release(void)
{
    int dev = 0;
    PRK_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lock(g_host_mu);
    if (static_cast<int>(g_host_ws.size()) > dev) {
        for (void*& p : g_host_ws[dev].d) {
            if (p) cudaFree(p);
            p = nullptr;
        }
        for (cudaStream_t& st : g_host_ws[dev].s) {
            if (st) cudaStreamDestroy(st);
            st = nullptr;
        }
        g_host_ws[dev].in_bytes = g_host_ws[dev].out_bytes = 0;
    }
    return PRK_OK;
}

}  // extern "C"
