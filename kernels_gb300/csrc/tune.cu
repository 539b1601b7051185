// The autotuner (prk_gb300_tune): times the candidate kernel configurations for a (pattern, radius,
// n, dtype) on scratch buffers and keeps the fastest in memory and in a JSON-lines cache file.
//
// Candidates, single grid: the tile kernels at temporal depth 1, 2, 4 and 8 and with the whole run
// in one launch, and the generic kernels. The tile kernels are the TMA ones, with tiles of 32 and of
// 64 rows (4 or 8 rows per thread), when the shape allows TMA (n a multiple of the vector width),
// else the plain-staged ones with tiles of 32 rows. Batched grids: the
// batched kernel at depth 1, 2, 4 and 8 and with the whole run in one launch. Every candidate
// computes the same bits (FP64) or stays within the FP32C bound, so the choice affects speed only.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <sys/stat.h>

#include "../../include/prk_gb300.h"
#include "prk_internal.cuh"
#include "stencil_tile.cuh"

namespace {

constexpr int64_t TUNE_NMAX = 8192;

std::mutex g_mu;
std::map<std::string, prk_gb300_tuning> g_cache;
bool g_loaded = false;

std::string cache_path()
{
    if (const char* p = std::getenv("PRK_GB300_TUNE_CACHE")) return p;
    if (const char* h = std::getenv("HOME")) {
        std::string dir = std::string(h) + "/.cache";
        mkdir(dir.c_str(), 0755);
        dir += "/prk_gb300";
        mkdir(dir.c_str(), 0755);
        return dir + "/tune.jsonl";
    }
    return "";
}

// {"key": "...", "depth": d, "kernel": k, "tile_rows": r, "tile_cols": c, "cols_per_thread": v, "seconds": s}
void load_cache()
{
    if (g_loaded) return;
    g_loaded = true;
    const std::string path = cache_path();
    if (path.empty()) return;
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return;
    char line[1024], key[512];
    while (std::fgets(line, sizeof line, f)) {
        prk_gb300_tuning t{};
        if (std::sscanf(line,
                        "{\"key\": \"%511[^\"]\", \"depth\": %d, \"kernel\": %d, \"tile_rows\": %d, \"tile_cols\": %d, "
                        "\"cols_per_thread\": %d, \"seconds\": %lf}",
                        key, &t.depth, &t.kernel, &t.tile_rows, &t.tile_cols, &t.cols_per_thread,
                        &t.seconds_per_application) == 7)
            g_cache[key] = t;
    }
    std::fclose(f);
}

void store_cache(const std::string& key, const prk_gb300_tuning& t)
{
    const std::string path = cache_path();
    if (path.empty()) return;
    FILE* f = std::fopen(path.c_str(), "a");
    if (!f) return;
    std::fprintf(f,
                 "{\"key\": \"%s\", \"depth\": %d, \"kernel\": %d, \"tile_rows\": %d, \"tile_cols\": %d, "
                 "\"cols_per_thread\": %d, \"seconds\": %.6e}\n",
                 key.c_str(), t.depth, t.kernel, t.tile_rows, t.tile_cols, t.cols_per_thread, t.seconds_per_application);
    std::fclose(f);
}

int64_t bucket(int64_t n)
{
    int64_t b = 64;
    while (b < n && b < TUNE_NMAX) b <<= 1;
    return b;
}

int err(int code, const char* msg) { return prk::record_error(code, msg); }

// Scratch buffers of one tuning run, freed on scope exit.
struct Scratch {
    void* p[3] = {nullptr, nullptr, nullptr};
    ~Scratch()
    {
        for (void* q : p)
            if (q) cudaFree(q);
    }
};

// Seconds per application of `apps` applications with the given flags (through prk_gb300_run).
int time_run(int pattern, int R, int64_t m, int dtype, int flags, Scratch& s, double* sec)
{
    if (int rc = prk_gb300_init(m, dtype, s.p[0], s.p[2], nullptr)) return rc;
    double el = 0.0;
    int fin = 0;
    const int apps = 16;
    if (int rc = prk_gb300_run(pattern, R, m, dtype, apps, s.p[0], s.p[1], s.p[2], flags, &el, &fin, nullptr)) return rc;
    *sec = el / apps;
    return PRK_OK;
}

int time_batch(int pattern, int R, int64_t m, int dtype, int depth, Scratch& s, double* sec)
{
    if (int rc = prk_gb300_init(m, dtype, s.p[0], s.p[2], nullptr)) return rc;
    prk_gb300_grid g{pattern, R, m, s.p[0], s.p[1], s.p[2]};
    prk_gb300_batch* b = nullptr;
    if (int rc = prk_gb300_batch_create(&g, 1, dtype, depth > 0 ? PRK_RUN_DEPTH(depth) : PRK_RUN_WHOLE, &b)) return rc;
    double el = 0.0;
    const int apps = 16;
    int rc = prk_gb300_batch_run(b, apps, 0, &el, nullptr);
    prk_gb300_batch_destroy(b);
    if (rc) return rc;
    *sec = el / apps;
    return PRK_OK;
}

}  // namespace

extern "C" int prk_gb300_tune(int pattern, int radius, int64_t n, int dtype, int flags, prk_gb300_tuning* result)
{
    if (!result) return err(PRK_ERR_ARG, "tune: null result");
    if (pattern != PRK_STAR && pattern != PRK_GRID) return err(PRK_ERR_ARG, "tune: bad pattern");
    if (dtype != PRK_FP64 && dtype != PRK_FP32C) return err(PRK_ERR_ARG, "tune: bad dtype");
    if (radius < 1 || radius > prk::RMAX || n < 1 || 2 * static_cast<int64_t>(radius) + 1 > n || n > prk::NMAX)
        return err(PRK_ERR_ARG, "tune: bad radius or n");
    const bool batch = (flags & PRK_TUNE_BATCH) != 0;
    const int vec = dtype == PRK_FP64 ? 2 : 4;
    const bool tma_shape = n % vec == 0 && n >= 8;
    int dev = 0;
    cudaDeviceProp prop{};
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
        return err(PRK_ERR_STATE, "tune: no CUDA device");
    char keybuf[512];
    std::snprintf(keybuf, sizeof keybuf, "%s|sm%d%d|%s|R%d|%s|n%lld|%s%s|v2", prop.name, prop.major, prop.minor,
                  pattern == PRK_STAR ? "star" : "grid", radius, dtype == PRK_FP64 ? "fp64" : "fp32c",
                  static_cast<long long>(bucket(n)), batch ? "batch" : "single", tma_shape ? "" : "|plain");
    const std::string key = keybuf;
    std::lock_guard<std::mutex> lock(g_mu);
    load_cache();
    if (!(flags & PRK_TUNE_FORCE)) {
        auto it = g_cache.find(key);
        if (it != g_cache.end()) {
            *result = it->second;
            result->from_cache = 1;
            return PRK_OK;
        }
    }

    // scratch grid: the caller's n up to TUNE_NMAX, keeping its TMA eligibility
    int64_t m = n < TUNE_NMAX ? n : TUNE_NMAX;
    if (tma_shape) m -= m % vec;
    Scratch s;
    const int64_t ib = prk_gb300_bytes(m, dtype, 0), ob = prk_gb300_bytes(m, dtype, 1);
    if (cudaMalloc(&s.p[0], ib) != cudaSuccess || cudaMalloc(&s.p[1], ib) != cudaSuccess || cudaMalloc(&s.p[2], ob) != cudaSuccess) {
        cudaGetLastError();
        return err(PRK_ERR_NOMEM, "tune: scratch allocation failed");
    }
    const int tw = dtype == PRK_FP64 ? prk::tile::Cfg<prk::FP64>::TW : prk::tile::Cfg<prk::FP32C>::TW;
    const int th = dtype == PRK_FP64 ? prk::tile::Cfg<prk::FP64>::TH : prk::tile::Cfg<prk::FP32C>::TH;
    const int cpt = dtype == PRK_FP64 ? prk::tile::Cfg<prk::FP64>::CPT : prk::tile::Cfg<prk::FP32C>::CPT;
    prk_gb300_tuning best{};
    best.seconds_per_application = 1e30;
    const int depths[4] = {1, 2, 4, 8};
    const int prev = prk_gb300_config(PRK_CFG_KERNEL, 0);
    int rc = PRK_OK;
    for (int tall = 0; tall < 2 && !rc; ++tall) {
        if (tall && (batch || !tma_shape)) break;  // the tall tiles exist for the TMA kernels only
        for (int d : depths) {
            double sec = 0.0;
            if (batch) {
                rc = time_batch(pattern, radius, m, dtype, d, s, &sec);
            } else {
                rc = time_run(pattern, radius, m, dtype, PRK_RUN_DEPTH(d) | (tall ? PRK_RUN_TALL : 0), s, &sec);
            }
            if (rc) break;
            if (sec < best.seconds_per_application) {
                best = prk_gb300_tuning{d, tma_shape ? 2 : 4, tall ? 64 : th, tw, cpt, sec, 0};
                if (batch) best.kernel = 3;
            }
        }
    }
    if (!rc && !batch) {  // the whole run in one launch
        double sec = 0.0;
        rc = time_run(pattern, radius, m, dtype, PRK_RUN_WHOLE, s, &sec);
        if (!rc && sec < best.seconds_per_application) best = prk_gb300_tuning{0, tma_shape ? 2 : 4, th, tw, cpt, sec, 0};
    }
    if (!rc && batch) {  // the batched kernel with the whole run in one launch
        double sec = 0.0;
        rc = time_batch(pattern, radius, m, dtype, 0, s, &sec);
        if (!rc && sec < best.seconds_per_application) best = prk_gb300_tuning{0, 3, th, tw, cpt, sec, 0};
    }
    if (!rc && !batch) {  // the generic kernels, depth 1
        double sec = 0.0;
        prk_gb300_config(PRK_CFG_KERNEL, 1);
        rc = time_run(pattern, radius, m, dtype, 0, s, &sec);
        prk_gb300_config(PRK_CFG_KERNEL, 0);
        if (!rc && sec < best.seconds_per_application) best = prk_gb300_tuning{1, 1, 16, 64, 1, sec, 0};
    }
    prk_gb300_config(PRK_CFG_KERNEL, prev);
    if (rc) return rc;
    g_cache[key] = best;
    store_cache(key, best);
    *result = best;
    return PRK_OK;
}
