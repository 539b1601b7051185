// stencil-gb300: the PRK stencil driver on the GB300 library.
//
// Same command line and the same report lines as the reference drivers
// (Cxx11/stencil-openmp.cc:81-262, Cxx11/stencil-cuda.cu:86-271):
//     stencil-gb300 <iterations> <n> [<tile> <star|grid> <radius>] [options]
// Options (after the positional arguments):
//     --dtype fp64|fp32c   storage/arithmetic form (default fp64)
//     --unfused            the reference structure: starR/gridR through the dispatch switch, then a
//                          separate in += 1 pass and a device synchronize every iteration
//     --graph              replay the timed iterations as one CUDA graph
//     --json               also print one JSON line with the results
// n is not capped at 46340: indices are 64-bit. The norm check is the reference's
// (|norm - 2(iterations+1)| <= 1e-8, stencil-openmp.cc:242-247).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>

#include "prk_gb300.h"
#include "prk_gb300_stencil.hpp"

namespace {

void nothing(const int n, const int t, const double* in, double* out)
{
    std::cout << "You are trying to use a stencil that does not exist.\n";
    if (n == 0 || t == 0) std::cout << in << out << std::endl;
    std::abort();
}

int die(const char* what)
{
    std::cout << "ERROR: " << what << ": " << prk_gb300_last_error() << std::endl;
    return 1;
}

}  // namespace

int main(int argc, char* argv[])
{
    std::cout << "Parallel Research Kernels" << std::endl;
    std::cout << "C++11/CUDA GB300 Stencil execution on 2D grid" << std::endl;

    int iterations = 0, radius = 2;
    long long n = 0, tile_size = 32;
    bool star = true, unfused = false, graph = false, json = false, tuned = false, whole = false;
    int dtype = PRK_FP64;
    int npos = 0;
    const char* pos[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    for (int a = 1; a < argc; ++a) {
        if (!std::strcmp(argv[a], "--unfused")) unfused = true;
        else if (!std::strcmp(argv[a], "--graph")) graph = true;
        else if (!std::strcmp(argv[a], "--tuned")) tuned = true;
        else if (!std::strcmp(argv[a], "--whole")) whole = true;
        else if (!std::strcmp(argv[a], "--json")) json = true;
        else if (!std::strcmp(argv[a], "--dtype") && a + 1 < argc) {
            const std::string d = argv[++a];
            if (d == "fp64") dtype = PRK_FP64;
            else if (d == "fp32c") dtype = PRK_FP32C;
            else {
                std::cout << "ERROR: --dtype must be fp64 or fp32c" << std::endl;
                return 1;
            }
        } else if (npos < 5) pos[npos++] = argv[a];
    }
    try {
        if (npos < 2) throw "Usage: <# iterations> <array dimension> [<tile_size> <star/grid> <radius>]";
        iterations = std::atoi(pos[0]);
        if (iterations < 1) throw "ERROR: iterations must be >= 1";
        n = std::atoll(pos[1]);
        if (n < 1) throw "ERROR: grid dimension must be positive";
        if (npos > 2) {
            tile_size = std::atoll(pos[2]);
            if (tile_size <= 0) tile_size = n;
            if (tile_size > n) tile_size = n;
        }
        if (npos > 3) star = std::string(pos[3]) != "grid";
        if (npos > 4) radius = std::atoi(pos[4]);
        if (radius < 1 || 2LL * radius + 1 > n) throw "ERROR: Stencil radius negative or too large";
        if (unfused && dtype != PRK_FP64) throw "ERROR: --unfused drives the double-precision starR/gridR operators only";
        if (unfused && (tuned || whole)) throw "ERROR: --tuned and --whole are fused forms";
    } catch (const char* e) {
        std::cout << e << std::endl;
        return 1;
    }

    int dev = 0;
    cudaDeviceProp prop{};
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        std::cout << "ERROR: no CUDA device" << std::endl;
        return 1;
    }
    std::cout << "Device                = " << prop.name << " (" << prop.multiProcessorCount << " SMs)" << std::endl;
    std::cout << "Number of iterations = " << iterations << std::endl;
    std::cout << "Grid size            = " << n << std::endl;
    std::cout << "Tile size            = " << tile_size << std::endl;
    std::cout << "Type of stencil      = " << (star ? "star" : "grid") << std::endl;
    std::cout << "Radius of stencil    = " << radius << std::endl;
    std::cout << "Data type            = " << (dtype == PRK_FP64 ? "fp64" : "fp32c") << std::endl;
    std::cout << "Update form          = " << (unfused ? "unfused (stencil, then in += 1)" : "fused ping-pong")
              << (graph ? ", CUDA graph" : "") << (tuned ? ", tuned" : "")
              << (whole ? ", whole run in one launch" : "") << std::endl;

    auto stencil = nothing;
    if (star) {
        switch (radius) {
        case 1: stencil = star1; break;
        case 2: stencil = star2; break;
        case 3: stencil = star3; break;
        case 4: stencil = star4; break;
        case 5: stencil = star5; break;
        }
    } else {
        switch (radius) {
        case 1: stencil = grid1; break;
        case 2: stencil = grid2; break;
        case 3: stencil = grid3; break;
        case 4: stencil = grid4; break;
        case 5: stencil = grid5; break;
        }
    }

    const int pattern = star ? PRK_STAR : PRK_GRID;
    const long long in_bytes = prk_gb300_bytes(n, dtype, 0), out_bytes = prk_gb300_bytes(n, dtype, 1);
    void *d_in = nullptr, *d_in2 = nullptr, *d_out = nullptr;
    if (cudaMalloc(&d_in, in_bytes) != cudaSuccess || (!unfused && cudaMalloc(&d_in2, in_bytes) != cudaSuccess) ||
        cudaMalloc(&d_out, out_bytes) != cudaSuccess) {
        std::cout << "ERROR: device allocation of " << (2 * in_bytes + out_bytes) << " bytes failed" << std::endl;
        return 1;
    }
    if (prk_gb300_init(n, dtype, d_in, d_out, nullptr) != PRK_OK) return die("init");

    double stencil_time = 0.0;
    if (unfused) {
        // The loop of Cxx11/stencil-cuda.cu:211-222 over the drop-in operators.
        auto t0 = std::chrono::steady_clock::now();
        for (int iter = 0; iter <= iterations; iter++) {
            if (iter == 1) t0 = std::chrono::steady_clock::now();
            stencil(static_cast<int>(n), static_cast<int>(tile_size), static_cast<const double*>(d_in),
                    static_cast<double*>(d_out));
            if (prk_gb300_add(n, dtype, d_in, nullptr) != PRK_OK) return die("add");
            if (cudaDeviceSynchronize() != cudaSuccess) return die("synchronize");
        }
        stencil_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    } else {
        int final_in = 0;
        const int flags = (graph ? PRK_RUN_GRAPH : 0) | (tuned ? PRK_RUN_TUNED : 0) | (whole ? PRK_RUN_WHOLE : 0);
        if (prk_gb300_run(pattern, radius, n, dtype, iterations, d_in, d_in2, d_out, flags, &stencil_time, &final_in,
                          nullptr) != PRK_OK)
            return die("run");
    }

    double norm = 0.0;
    if (prk_gb300_norm(radius, n, dtype, d_out, &norm, nullptr) != PRK_OK) return die("norm");
    cudaFree(d_in);
    if (d_in2) cudaFree(d_in2);
    cudaFree(d_out);

    const double epsilon = 1.0e-8;
    const double reference_norm = 2. * (iterations + 1.);
    const double flops = prk_gb300_flops(pattern, radius, n);
    const double avgtime = stencil_time / iterations;
    int rc = 0;
    if (std::fabs(norm - reference_norm) > epsilon) {
        std::cout << "ERROR: L1 norm = " << norm << " Reference L1 norm = " << reference_norm << std::endl;
        rc = 1;
    } else {
        std::cout << "Solution validates" << std::endl;
        std::cout << "L1 norm = " << norm << " Reference L1 norm = " << reference_norm << std::endl;
        std::cout << "Rate (MFlops/s): " << 1.0e-6 * flops / avgtime << " Avg time (s): " << avgtime << std::endl;
    }
    if (json) {
        std::printf("{\"n\": %lld, \"iterations\": %d, \"pattern\": \"%s\", \"radius\": %d, \"dtype\": \"%s\", "
                    "\"unfused\": %s, \"graph\": %s, \"norm\": %.17g, \"validates\": %s, \"avg_time_s\": %.9g, "
                    "\"gflops\": %.6g}\n",
                    n, iterations, star ? "star" : "grid", radius, dtype == PRK_FP64 ? "fp64" : "fp32c",
                    unfused ? "true" : "false", graph ? "true" : "false", norm, rc == 0 ? "true" : "false", avgtime,
                    1.0e-9 * flops / avgtime);
    }
    return rc;
}
