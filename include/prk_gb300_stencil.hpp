// prk_gb300_stencil.hpp - drop-in C++ stencil operators over the C ABI.
//
// The reference drivers pick an operator through a switch into a function pointer
// (Cxx11/stencil-openmp.cc:154-171) whose signature is
//     void starR(const int n, const int t, const double* in, double* out)   (Cxx11/stencil_openmp.hpp:1)
// The functions below keep those names and that signature, so a driver with the reference's
// structure dispatches to the GB300 kernels through the same switch. Differences:
//   - in and out are DEVICE pointers (as in Cxx11/stencil-cuda.cu:206-216), double[n*n];
//   - t, the CPU tile size, is accepted and ignored: the GPU tiling is the library's;
//   - the call is asynchronous on the legacy default stream, like a kernel launch;
//   - an error prints the library's message and calls std::abort(), as prk::check does
//     (Cxx11/prk_cuda.h:40-46).
// The in += 1 sweep stays with the caller (prk_gb300_add), as in the reference drivers.
#ifndef PRK_GB300_STENCIL_HPP
#define PRK_GB300_STENCIL_HPP

#include <cstdio>
#include <cstdlib>

#include "prk_gb300.h"

namespace prk_gb300 {

inline void check(int rc)
{
    if (rc != PRK_OK) {
        std::fprintf(stderr, "prk_gb300: %s\n", prk_gb300_last_error());
        std::abort();
    }
}

template <int PATTERN, int R>
inline void apply(const int n, const int /*t*/, const double* in, double* out)
{
    check(prk_gb300_stencil(PATTERN, R, n, PRK_FP64, in, nullptr, out, nullptr));
}

}  // namespace prk_gb300

inline void star1(const int n, const int t, const double* in, double* out) { prk_gb300::apply<PRK_STAR, 1>(n, t, in, out); }
inline void star2(const int n, const int t, const double* in, double* out) { prk_gb300::apply<PRK_STAR, 2>(n, t, in, out); }
inline void star3(const int n, const int t, const double* in, double* out) { prk_gb300::apply<PRK_STAR, 3>(n, t, in, out); }
inline void star4(const int n, const int t, const double* in, double* out) { prk_gb300::apply<PRK_STAR, 4>(n, t, in, out); }
inline void star5(const int n, const int t, const double* in, double* out) { prk_gb300::apply<PRK_STAR, 5>(n, t, in, out); }
inline void grid1(const int n, const int t, const double* in, double* out) { prk_gb300::apply<PRK_GRID, 1>(n, t, in, out); }
inline void grid2(const int n, const int t, const double* in, double* out) { prk_gb300::apply<PRK_GRID, 2>(n, t, in, out); }
inline void grid3(const int n, const int t, const double* in, double* out) { prk_gb300::apply<PRK_GRID, 3>(n, t, in, out); }
inline void grid4(const int n, const int t, const double* in, double* out) { prk_gb300::apply<PRK_GRID, 4>(n, t, in, out); }
inline void grid5(const int n, const int t, const double* in, double* out) { prk_gb300::apply<PRK_GRID, 5>(n, t, in, out); }

#endif  // PRK_GB300_STENCIL_HPP
