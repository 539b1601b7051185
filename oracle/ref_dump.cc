// Dump harness around the reference's own serial stencil operator (test infrastructure only).
//
// It includes the reference headers where they lie (Cxx11/prk_util.h, Cxx11/stencil_seq.hpp) and
// repeats the serial driver's run (Cxx11/stencil.cc:168-191: init in=i+j, out=0, iterations+1
// applications each followed by in += 1), then writes the raw little-endian `out` array to a file
// and prints the L1 norm as stencil.cc:197-204 computes it, in hex and decimal.
//
//   ref_dump <iterations> <n> <tile> <star|grid> <radius> <out.bin>

#include "prk_util.h"
#include "stencil_seq.hpp"

#include <cstdio>

int main(int argc, char* argv[])
{
    if (argc != 7) {
        std::fprintf(stderr, "usage: ref_dump <iterations> <n> <tile> <star|grid> <radius> <out.bin>\n");
        return 2;
    }
    const int iterations = std::atoi(argv[1]);
    const int n = std::atoi(argv[2]);
    int tile = std::atoi(argv[3]);
    const bool star = std::string(argv[4]) != "grid";
    const int radius = std::atoi(argv[5]);
    if (iterations < 1 || n < 1 || n > prk::get_max_matrix_size() || radius < 1 || radius > 5 || 2 * radius + 1 > n) {
        std::fprintf(stderr, "bad arguments\n");
        return 2;
    }
    if (tile <= 0 || tile > n) tile = n;

    using fn = void (*)(const int, const int, prk::vector<double>&, prk::vector<double>&);
    const fn stars[6] = {nullptr, star1, star2, star3, star4, star5};
    const fn grids[6] = {nullptr, grid1, grid2, grid3, grid4, grid5};
    const fn stencil = star ? stars[radius] : grids[radius];

    prk::vector<double> in(n * n);
    prk::vector<double> out(n * n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            in[i * n + j] = static_cast<double>(i + j);
            out[i * n + j] = 0.0;
        }
    for (int iter = 0; iter <= iterations; iter++) {
        stencil(n, tile, in, out);
        for (auto& c : in) c += 1.0;
    }

    double norm = 0.0;
    for (int i = radius; i < n - radius; i++)
        for (int j = radius; j < n - radius; j++) norm += prk::abs(out[i * n + j]);
    norm /= static_cast<double>(n - 2 * radius) * static_cast<double>(n - 2 * radius);

    std::FILE* f = std::fopen(argv[6], "wb");
    if (!f) return 3;
    const size_t wrote = std::fwrite(&out[0], sizeof(double), static_cast<size_t>(n) * n, f);
    std::fclose(f);
    if (wrote != static_cast<size_t>(n) * n) return 3;
    std::printf("norm %a %.17g\n", norm, norm);
    return 0;
}
