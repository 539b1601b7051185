// Host side of the batched grids (prk_gb300_batch_*): device tables, the work-queue slots, the
// launch sequence of a run and its CUDA graph.
#include <algorithm>
#include <cstdio>
#include <map>
#include <memory>
#include <vector>

#include "../../include/prk_gb300.h"
#include "batch_kernel.cuh"
#include "prk_internal.cuh"

namespace {

using prk::batch::GridDesc;

int err(int code, const char* msg) { return prk::record_error(code, msg); }

int cuda_err(cudaError_t e, const char* what)
{
    char msg[256];
    std::snprintf(msg, sizeof msg, "%s: %s", what, cudaGetErrorString(e));
    return prk::record_error(static_cast<int>(e), msg);
}

// Grids advanced by one kernel sequence: all of one kernel family (prk::batch::family_of) and one
// temporal depth.
struct Group {
    int family = 0;
    int depth = 1;                     // applications per launch; 0: the rest of the run in one launch
    std::vector<int> members;          // indices into the batch's grid list
    GridDesc* d_desc = nullptr;        // device descriptors
    int64_t* d_off = nullptr;          // device tile offsets (members + 1)
    int64_t total = 0;                 // tiles over all members
    int ctas = 0;                      // persistent CTAs per launch of this group's kernel
};

}  // namespace

struct prk_gb300_batch {
    int dtype = PRK_FP64;
    std::vector<prk_gb300_grid> grids;
    std::vector<int> final_in;         // per grid, after the last run
    std::vector<Group> groups;
    unsigned long long* d_queue = nullptr;  // one work counter per launch of a run
    int queue_slots = 0;
    std::vector<cudaStream_t> streams;  // one per group: the groups' launches run side by side
    std::vector<cudaEvent_t> joins;     // one per group: its last launch done
    cudaEvent_t fork = nullptr;
    std::map<int, cudaGraphExec_t> graphs;  // per iteration count
    int device = 0;
};

namespace {

int vec_width(int dtype) { return dtype == PRK_FP64 ? 2 : 4; }

int tiles_of(int64_t n, int dtype, int* tx)
{
    const int tw = dtype == PRK_FP64 ? prk::tile::Cfg<prk::FP64>::TW : prk::tile::Cfg<prk::FP32C>::TW;
    const int th = dtype == PRK_FP64 ? prk::tile::Cfg<prk::FP64>::TH : prk::tile::Cfg<prk::FP32C>::TH;
    *tx = static_cast<int>((n + tw - 1) / tw);
    return static_cast<int>(((n + th - 1) / th) * *tx);
}

// Device descriptor and tile-offset tables for a list of grids.
int build_tables(prk_gb300_batch* b, const std::vector<int>& members, GridDesc** d_desc, int64_t** d_off, int64_t* total)
{
    std::vector<GridDesc> desc(members.size());
    std::vector<int64_t> off(members.size() + 1, 0);
    for (size_t k = 0; k < members.size(); ++k) {
        const prk_gb300_grid& g = b->grids[members[k]];
        GridDesc& d = desc[k];
        d.n = g.n;
        d.in[0] = g.in_a;
        d.in[1] = g.in_b;
        d.out = g.out;
        d.pattern = g.pattern;
        d.R = g.radius;
        d.tiles = tiles_of(g.n, b->dtype, &d.tiles_x);
        auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
        d.vec_ok = (g.n % vec_width(b->dtype) == 0) && al16(g.in_a) && al16(g.in_b) && al16(g.out);
        off[k + 1] = off[k] + d.tiles;
    }
    *total = off.back();
    cudaError_t e;
    if ((e = cudaMalloc(d_desc, sizeof(GridDesc) * std::max<size_t>(desc.size(), 1))) != cudaSuccess ||
        (e = cudaMalloc(d_off, sizeof(int64_t) * off.size())) != cudaSuccess) {
        cudaGetLastError();
        return err(PRK_ERR_NOMEM, "batch: device table allocation failed");
    }
    if ((e = cudaMemcpy(*d_desc, desc.data(), sizeof(GridDesc) * desc.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(*d_off, off.data(), sizeof(int64_t) * off.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_err(e, "batch: table upload");
    return PRK_OK;
}

// A launch of group g's kernel: steps 1, 2, 4 or 8, a launch of that depth; steps 0, one launch of
// `apps` applications.
cudaError_t launch_group(const prk_gb300_batch* b, const Group& g, int steps, int slot, int parity, cudaStream_t s,
                         int apps = 0)
{
    prk::batch::Launch L{g.d_desc, g.d_off, static_cast<int>(g.members.size()), g.total, b->d_queue + slot, parity,
                         g.ctas, s, apps};
    return prk::batch::launch_family(b->dtype, g.family, steps, L);
}

// Applications of a group's next launch with `left` to go: the whole rest for depth 0, else the
// group depth, the remainder in powers of two.
int next_apps(int depth, int left)
{
    if (depth == 0) return left;
    int d = depth;
    while (d > left) d >>= 1;
    return d;
}

int launches_of(const prk_gb300_batch* b, int iterations)
{
    int total = 0;
    for (const Group& g : b->groups)
        total += g.depth == 0 ? 1 : (iterations + g.depth - 1) / g.depth + 2;  // remainder split in powers of 2
    return total;
}

// The timed part of a run: every group's launches for `iterations` applications, each group on its
// own stream forked from and joined back into `s` (inside a capture this makes parallel branches of
// the graph), so that different families' kernels share the GPU. Queue slots from the number of
// groups on (the slots below are the warm-up's); group parities start at 1 (after the warm-up).
int enqueue_timed(prk_gb300_batch* b, int iterations, cudaStream_t s, std::vector<int>* parity_out)
{
    int slot = static_cast<int>(b->groups.size());
    parity_out->assign(b->groups.size(), 1);
    if (cudaError_t e = cudaEventRecord(b->fork, s)) return cuda_err(e, "cudaEventRecord");
    for (size_t gi = 0; gi < b->groups.size(); ++gi) {
        Group& g = b->groups[gi];
        cudaStream_t gs = b->streams[gi];
        if (cudaError_t e = cudaStreamWaitEvent(gs, b->fork, 0)) return cuda_err(e, "cudaStreamWaitEvent");
        int parity = 1, left = iterations;
        while (left > 0) {
            const int d = next_apps(g.depth, left);
            if (slot >= b->queue_slots) return err(PRK_ERR_STATE, "batch: more launches than queue slots");
            cudaError_t e = launch_group(b, g, g.depth == 0 ? 0 : d, slot++, parity, gs, d);
            if (e != cudaSuccess) return cuda_err(e, "batch launch");
            parity ^= 1;
            left -= d;
        }
        (*parity_out)[gi] = parity;
        if (cudaError_t e = cudaEventRecord(b->joins[gi], gs)) return cuda_err(e, "cudaEventRecord");
        if (cudaError_t e = cudaStreamWaitEvent(s, b->joins[gi], 0)) return cuda_err(e, "cudaStreamWaitEvent");
    }
    return PRK_OK;
}

}  // namespace

extern "C" {

int prk_gb300_batch_create(const prk_gb300_grid* grids, int count, int dtype, int flags, prk_gb300_batch** out)
{
    if (!out) return err(PRK_ERR_ARG, "batch: null output handle");
    *out = nullptr;
    if (!grids || count < 1) return err(PRK_ERR_ARG, "batch: need at least one grid");
    if (dtype != PRK_FP64 && dtype != PRK_FP32C) return err(PRK_ERR_ARG, "batch: dtype is not PRK_FP64 or PRK_FP32C");
    int depth = (flags >> 8) & 0xFF;
    if (depth == 0) depth = 1;
    if (!prk::tma_depth_ok(depth)) return err(PRK_ERR_ARG, "batch: temporal depth is not 1, 2, 4 or 8");
    if (flags & PRK_RUN_WHOLE) depth = 0;
    for (int k = 0; k < count; ++k) {
        const prk_gb300_grid& g = grids[k];
        if ((g.pattern != PRK_STAR && g.pattern != PRK_GRID) || g.radius < 1 || g.radius > prk::RMAX || g.n < 1 ||
            2 * static_cast<int64_t>(g.radius) + 1 > g.n || g.n > prk::NMAX)
            return err(PRK_ERR_ARG, "batch: a grid has a bad pattern, radius or n");
        if (!g.in_a || !g.in_b || !g.out) return err(PRK_ERR_ARG, "batch: a grid has a null buffer");
    }
    std::unique_ptr<prk_gb300_batch> b(new prk_gb300_batch);
    b->dtype = dtype;
    b->grids.assign(grids, grids + count);
    b->final_in.assign(count, 0);
    if (cudaError_t e = cudaGetDevice(&b->device)) return cuda_err(e, "cudaGetDevice");

    // group by kernel family and temporal depth (tuned per grid, or one fixed depth)
    std::map<std::pair<int, int>, std::vector<int>> by_key;
    for (int k = 0; k < count; ++k) {
        int d = depth;
        if (flags & PRK_BATCH_TUNED) {
            prk_gb300_tuning t{};
            if (int rc = prk_gb300_tune(grids[k].pattern, grids[k].radius, grids[k].n, dtype, PRK_TUNE_BATCH, &t)) return rc;
            d = t.depth;
        }
        by_key[{prk::batch::family_of(dtype, grids[k].pattern, grids[k].radius), d}].push_back(k);
    }
    int sms = 0;
    if (cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device)) return cuda_err(e, "device query");
    for (auto& kv : by_key) {
        Group g;
        g.family = kv.first.first;
        g.depth = kv.first.second;
        g.members = kv.second;
        g.ctas = sms * std::max(prk::batch::ctas_per_sm_family(dtype, g.family, g.depth), 1);
        const int rc = build_tables(b.get(), g.members, &g.d_desc, &g.d_off, &g.total);
        b->groups.push_back(std::move(g));
        if (rc) {
            prk_gb300_batch_destroy(b.release());  // frees what was made so far
            return rc;
        }
    }
    auto fail_free = [&](int rc) {
        prk_gb300_batch_destroy(b.release());
        return rc;
    };
    for (size_t gi = 0; gi < b->groups.size(); ++gi) {
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        if (cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) return fail_free(cuda_err(e, "cudaStreamCreate"));
        b->streams.push_back(st);
        if (cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) return fail_free(cuda_err(e, "cudaEventCreate"));
        b->joins.push_back(ev);
    }
    if (cudaError_t e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) return fail_free(cuda_err(e, "cudaEventCreate"));
    b->queue_slots = 4096;
    if (cudaMalloc(&b->d_queue, sizeof(unsigned long long) * b->queue_slots) != cudaSuccess) {
        cudaGetLastError();
        return fail_free(err(PRK_ERR_NOMEM, "batch: queue allocation failed"));
    }
    *out = b.release();
    return PRK_OK;
}

int prk_gb300_batch_run(prk_gb300_batch* b, int iterations, int flags, double* elapsed_s, void* stream)
{
    if (!b) return err(PRK_ERR_ARG, "batch: null handle");
    if (iterations < 1) return err(PRK_ERR_ARG, "iterations must be >= 1");
    if (launches_of(b, iterations) + static_cast<int>(b->groups.size()) > b->queue_slots)
        return err(PRK_ERR_LIMIT, "batch: too many launches for one run");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaStream_t own = nullptr;
    const bool graph = (flags & PRK_RUN_GRAPH) != 0;
    if (graph && !s) {
        if (cudaError_t e = cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking)) return cuda_err(e, "cudaStreamCreate");
        s = own;
        cudaDeviceSynchronize();  // order the private stream after prior legacy-stream work
    }
    int rc = PRK_OK;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<int> parity;
    do {
        cudaError_t e;
        if ((e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) { rc = cuda_err(e, "cudaEventCreate"); break; }
        // application 0 (untimed warm-up): one depth-1 launch per group, queue slots 0 .. groups - 1
        const int ng = static_cast<int>(b->groups.size());
        if ((e = cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned long long) * b->queue_slots, s)) != cudaSuccess) { rc = cuda_err(e, "queue reset"); break; }
        for (int gi = 0; gi < ng && e == cudaSuccess; ++gi) e = launch_group(b, b->groups[gi], 1, gi, 0, s);
        if (e != cudaSuccess) { rc = cuda_err(e, "batch warm-up launch"); break; }
        if (graph) {
            cudaGraphExec_t ge = nullptr;
            auto it = b->graphs.find(iterations);
            if (it == b->graphs.end()) {
                cudaGraph_t g = nullptr;
                if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) { rc = cuda_err(e, "cudaStreamBeginCapture"); break; }
                rc = cudaMemsetAsync(b->d_queue + ng, 0, sizeof(unsigned long long) * (b->queue_slots - ng), s) == cudaSuccess
                         ? enqueue_timed(b, iterations, s, &parity) : err(PRK_ERR_STATE, "queue reset during capture");
                cudaError_t ec = cudaStreamEndCapture(s, &g);
                if (rc != PRK_OK) { if (g) cudaGraphDestroy(g); break; }
                if (ec != cudaSuccess) { rc = cuda_err(ec, "cudaStreamEndCapture"); break; }
                e = cudaGraphInstantiate(&ge, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) { rc = cuda_err(e, "cudaGraphInstantiate"); break; }
                if ((e = cudaGraphUpload(ge, s)) != cudaSuccess) { rc = cuda_err(e, "cudaGraphUpload"); cudaGraphExecDestroy(ge); break; }
                b->graphs[iterations] = ge;
            } else {
                ge = it->second;
                parity.assign(b->groups.size(), 1);
                for (size_t gi = 0; gi < b->groups.size(); ++gi) {  // same launch sequence as captured
                    int p = 1, left = iterations;
                    while (left > 0) {
                        p ^= 1;
                        left -= next_apps(b->groups[gi].depth, left);
                    }
                    parity[gi] = p;
                }
            }
            cudaEventRecord(e0, s);
            if ((e = cudaGraphLaunch(ge, s)) != cudaSuccess) { rc = cuda_err(e, "cudaGraphLaunch"); break; }
            cudaEventRecord(e1, s);
        } else {
            cudaEventRecord(e0, s);
            if ((rc = enqueue_timed(b, iterations, s, &parity)) != PRK_OK) break;
            cudaEventRecord(e1, s);
        }
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) { rc = cuda_err(e, "batch run"); break; }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (elapsed_s) *elapsed_s = ms * 1e-3;
        for (size_t gi = 0; gi < b->groups.size(); ++gi)
            for (int k : b->groups[gi].members) b->final_in[k] = parity[gi];
        rc = prk_gb300_status();
    } while (false);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (own) {
        cudaStreamSynchronize(own);
        cudaStreamDestroy(own);
    }
    return rc;
}

int prk_gb300_batch_final_in(const prk_gb300_batch* b, int index)
{
    if (!b || index < 0 || index >= static_cast<int>(b->grids.size())) return PRK_ERR_ARG;
    return b->final_in[index];
}

int prk_gb300_batch_norms(prk_gb300_batch* b, double* norms, void* stream)
{
    if (!b || !norms) return err(PRK_ERR_ARG, "batch: null handle or norms");
    for (size_t k = 0; k < b->grids.size(); ++k) {
        const prk_gb300_grid& g = b->grids[k];
        if (int rc = prk_gb300_norm(g.radius, g.n, b->dtype, g.out, &norms[k], stream)) return rc;
    }
    return PRK_OK;
}

int prk_gb300_batch_launches(const prk_gb300_batch* b, int iterations)
{
    if (!b || iterations < 1) return PRK_ERR_ARG;
    int total = 0;
    for (const Group& g : b->groups) {
        int left = iterations;
        while (left > 0) {
            ++total;
            left -= next_apps(g.depth, left);
        }
    }
    return total;
}

int prk_gb300_batch_destroy(prk_gb300_batch* b)
{
    if (!b) return PRK_OK;
    cudaDeviceSynchronize();
    for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
    for (Group& g : b->groups) {
        cudaFree(g.d_desc);
        cudaFree(g.d_off);
    }
    for (cudaStream_t st : b->streams) cudaStreamDestroy(st);
    for (cudaEvent_t ev : b->joins) cudaEventDestroy(ev);
    if (b->fork) cudaEventDestroy(b->fork);
    cudaFree(b->d_queue);
    delete b;
    return PRK_OK;
}

}  // extern "C"
