// The two PRK kernels that share the stencil's bandwidth roofline: nstream (the STREAM triad,
// Cxx11/nstream-cuda.cu:68-76) and transpose (Cxx11/transpose-cuda.cu:65-123). One application per
// call, as the reference's timed loop makes it; binary64 with every product and sum rounded on its
// own, in the reference's order, so the results are those of its strict evaluation.
//
// transpose's A += 1 has an exact integer form for positive whole numbers (inc_exact,
// prk_arith.cuh); B += A^T stays a binary64 add.
//
// nstream's three binary64 operations per element keep this GPU's binary64 pipe 82% busy at 68% of
// DRAM peak, so it has a certified exact route: where the operands are whole numbers below 2^20
// and the scalar a whole number of magnitude <= 8, every binary64 operation of the reference's
// sequence is exact, and so are the same operations in FP32 (all partial results below 2^24). The
// operands are checked and converted with a few integer operations, the result converted back by
// rebiasing its exponent. An element outside the bounds takes the binary64 instructions. -0 is
// never certified, so the sign of a zero comes out as binary64 gives it.
//
// nstream    A[i] += B[i] + scalar * C[i]: 32 B of HBM traffic per element (read A, B, C, write
//            A). A grid-stride loop in which each block takes 1024 consecutive 16-byte vectors
//            of each array per trip, four per thread, all twelve loads issued before any arithmetic (scalar head and tail where the pointers or the
//            length are not 16-byte aligned), grid sized to the SM count.
// transpose  B += A^T, then A += 1 (the accumulate form): 32 B per element (read and write A, read
//            and write B). 64 x 64 tiles of A staged in shared memory with one column of padding.
//            A thread issues all its loads at once: its A rows as 16-byte vectors and its strip
//            of the transposed B tile; A goes back (+1) as 16-byte vectors and B along its rows
//            while the tile is read down its columns, free of bank conflicts.
#include <cstdint>

#include "../../include/prk_gb300.h"
#include "prk_arith.cuh"
#include "prk_internal.cuh"

namespace prk {
namespace {

constexpr int NS_THREADS = 256;

// f == d for +0 or a whole number 1 <= |d| < 2^20; false otherwise. Integer operations on the
// encoding and one FP32 rounding test, no binary64 instruction.
__device__ __forceinline__ bool small_whole(double d, float& f)
{
    const uint64_t b = static_cast<uint64_t>(__double_as_longlong(d));
    const uint32_t hi = static_cast<uint32_t>(b >> 32), lo = static_cast<uint32_t>(b);
    const uint32_t e = (hi >> 20) & 0x7FFu;
    const bool small = e - 1023u < 20u && (lo & 0x1FFFFFFFu) == 0u;
    f = __uint_as_float((hi & 0x80000000u) | (((hi & 0x7FFFFFFFu) - (896u << 20)) << 3) | (lo >> 29));
    const float r = __fsub_rn(__fadd_rn(f, 12582912.0f), 12582912.0f);  // nearest whole number, |f| < 2^22
    if (b == 0) f = 0.0f;
    return b == 0 || (small && r == f);
}

// binary64 encoding of a whole-number f, |f| < 2^24: exponent rebias and a mantissa shift.
__device__ __forceinline__ double widen(float f)
{
    const uint32_t u = __float_as_uint(f);
    const uint64_t mag = u & 0x7FFFFFFFu;
    const uint64_t d = (static_cast<uint64_t>(u & 0x80000000u) << 32) | ((mag + (896ull << 23)) << 29);
    return __longlong_as_double(static_cast<long long>(mag == 0 ? 0ull : d));
}

// nstream for one element. EXACT: the scalar is a whole number with |s| <= 8 (checked on the
// host); with |a|, |b|, |c| < 2^20 whole numbers, |s*c| < 2^23 and the sums stay below 2^24.
template <bool EXACT>
__device__ __forceinline__ double triad(double a, double b, double c, double scalar, float sf)
{
    if (EXACT) {
        float fa, fb, fc;
        const bool ok = small_whole(a, fa) & small_whole(b, fb) & small_whole(c, fc);
        if (ok) return widen(__fadd_rn(fa, __fadd_rn(fb, __fmul_rn(sf, fc))));
    }
    return __dadd_rn(a, __dadd_rn(b, __dmul_rn(scalar, c)));
}

template <bool EXACT>
__global__ void __launch_bounds__(NS_THREADS) k_nstream(int64_t head, int64_t nvec, int64_t length, double scalar,
                                                         float sf, double* __restrict__ A,
                                                         const double* __restrict__ B, const double* __restrict__ C)
{
    const int64_t stride = static_cast<int64_t>(gridDim.x) * NS_THREADS;
    const int64_t t = static_cast<int64_t>(blockIdx.x) * NS_THREADS + threadIdx.x;
    // 16-byte vectors from element `head` on (A, B and C share their offset from a 16-byte boundary)
    double2* A2 = reinterpret_cast<double2*>(A + head);
    const double2* B2 = reinterpret_cast<const double2*>(B + head);
    const double2* C2 = reinterpret_cast<const double2*>(C + head);
    constexpr int U = 4;  // vectors per thread per trip; a block's trip covers U * 256 consecutive vectors
    for (int64_t v0 = static_cast<int64_t>(blockIdx.x) * U * NS_THREADS + threadIdx.x; v0 < nvec; v0 += U * stride) {
        double2 a[U], b[U], c[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t v = v0 + u * NS_THREADS;
            if (v < nvec) {
                a[u] = A2[v];
                b[u] = B2[v];
                c[u] = C2[v];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t v = v0 + u * NS_THREADS;
            if (v < nvec) {
                a[u].x = triad<EXACT>(a[u].x, b[u].x, c[u].x, scalar, sf);
                a[u].y = triad<EXACT>(a[u].y, b[u].y, c[u].y, scalar, sf);
                A2[v] = a[u];
            }
        }
    }
    // the scalar head (at most one element) and tail
    const int64_t tail0 = head + 2 * nvec;
    for (int64_t i = t; i < head + (length - tail0); i += stride) {
        const int64_t k = i < head ? i : tail0 + (i - head);
        A[k] = triad<EXACT>(A[k], B[k], C[k], scalar, sf);
    }
}

constexpr int TT = 64;           // transpose tile edge
constexpr int TP = TT + 1;       // padded row length of the shared tile
constexpr int TR_THREADS = 256;  // 8 warps

__global__ void __launch_bounds__(TR_THREADS, 2) k_transpose(int64_t order, double* __restrict__ A,
                                                          double* __restrict__ B, int vec)
{
    __shared__ double tile[TT * TP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t x0 = static_cast<int64_t>(blockIdx.x) * TT;  // columns of A, rows of B
    const int64_t y0 = static_cast<int64_t>(blockIdx.y) * TT;  // rows of A, columns of B
    constexpr int RPW = TT / 8;  // rows per warp
    // loads first: A rows y0 + warp + 8 q (lane owns columns 2 lane, 2 lane + 1) and the B strip,
    // rows x0 + warp + 8 q, columns y0 + lane and y0 + 32 + lane
    double a0[RPW], a1[RPW], b[RPW][2];
#pragma unroll
    for (int q = 0; q < RPW; ++q) {
        const int rr = warp + 8 * q;
        const int64_t y = y0 + rr, x = x0 + 2 * lane;
        a0[q] = 0.0;
        a1[q] = 0.0;
        if (y < order) {
            const double* p = A + y * order + x;
            if (vec && x + 1 < order) {
                const double2 v = *reinterpret_cast<const double2*>(p);
                a0[q] = v.x;
                a1[q] = v.y;
            } else {
                if (x < order) a0[q] = p[0];
                if (x + 1 < order) a1[q] = p[1];
            }
        }
        const int64_t bx = x0 + rr;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int64_t by = y0 + lane + 32 * h;
            b[q][h] = (bx < order && by < order) ? B[bx * order + by] : 0.0;
        }
    }
    // the tile, and A + 1 back
#pragma unroll
    for (int q = 0; q < RPW; ++q) {
        const int rr = warp + 8 * q;
        tile[rr * TP + 2 * lane] = a0[q];
        tile[rr * TP + 2 * lane + 1] = a1[q];
        const int64_t y = y0 + rr, x = x0 + 2 * lane;
        if (y < order) {
            double* p = A + y * order + x;
            if (vec && x + 1 < order) {
                *reinterpret_cast<double2*>(p) = make_double2(inc_exact(a0[q]), inc_exact(a1[q]));
            } else {
                if (x < order) p[0] = inc_exact(a0[q]);
                if (x + 1 < order) p[1] = inc_exact(a1[q]);
            }
        }
    }
    __syncthreads();
    // B[x][y] += A[y][x] = tile[y - y0][x - x0]
#pragma unroll
    for (int q = 0; q < RPW; ++q) {
        const int rr = warp + 8 * q;
        const int64_t bx = x0 + rr;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int c = lane + 32 * h;
            const int64_t by = y0 + c;
            if (bx < order && by < order) B[bx * order + by] = __dadd_rn(b[q][h], tile[c * TP + rr]);
        }
    }
}

int sms()
{
    static int count = 0;
    if (!count) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || count < 1)
            count = 132;
    }
    return count;
}

bool overlap(const void* a, int64_t an, const void* b, int64_t bn)
{
    const auto pa = reinterpret_cast<uintptr_t>(a), pb = reinterpret_cast<uintptr_t>(b);
    return pa < pb + static_cast<uintptr_t>(bn) && pb < pa + static_cast<uintptr_t>(an);
}

}  // namespace
}  // namespace prk

extern "C" {

int prk_gb300_nstream(int64_t length, double scalar, double* A, const double* B, const double* C, void* stream)
{
    if (length < 1) return prk::record_error(PRK_ERR_ARG, "nstream: length must be >= 1");
    if (!A || !B || !C) return prk::record_error(PRK_ERR_ARG, "nstream: null vector");
    const int64_t bytes = length * 8;
    if (prk::overlap(A, bytes, B, bytes) || prk::overlap(A, bytes, C, bytes))
        return prk::record_error(PRK_ERR_ARG, "nstream: A overlaps B or C");
    const auto off = [](const void* p) { return reinterpret_cast<uintptr_t>(p) & 15u; };
    int64_t head = 0, nvec = 0;
    if (off(A) == off(B) && off(A) == off(C) && off(A) % 8 == 0) {
        head = off(A) ? 1 : 0;
        if (head > length) head = length;
        nvec = (length - head) / 2;
    }
    const int64_t work = nvec > 0 ? nvec : length;
    int64_t blocks = (work + prk::NS_THREADS - 1) / prk::NS_THREADS;
    const int64_t cap = static_cast<int64_t>(prk::sms()) * 8;
    if (blocks > cap) blocks = cap;
    // the exact route needs a whole-number scalar |s| <= 8
    const bool exact = scalar >= -8.0 && scalar <= 8.0 && scalar == static_cast<double>(static_cast<int>(scalar));
    const float sf = exact ? static_cast<float>(scalar) : 0.0f;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (exact)
        prk::k_nstream<true><<<static_cast<unsigned>(blocks), prk::NS_THREADS, 0, st>>>(head, nvec, length, scalar, sf, A, B, C);
    else
        prk::k_nstream<false><<<static_cast<unsigned>(blocks), prk::NS_THREADS, 0, st>>>(head, nvec, length, scalar, sf, A, B, C);
    if (cudaError_t e = cudaGetLastError()) return prk::record_error(PRK_ERR_STATE, cudaGetErrorString(e));
    return PRK_OK;
}

int prk_gb300_transpose(int64_t order, double* A, double* B, void* stream)
{
    if (order < 1) return prk::record_error(PRK_ERR_ARG, "transpose: order must be >= 1");
    if (!A || !B) return prk::record_error(PRK_ERR_ARG, "transpose: null matrix");
    const int64_t tiles = (order + prk::TT - 1) / prk::TT;
    if (tiles > 65535) return prk::record_error(PRK_ERR_LIMIT, "transpose: order above 65535 * 64");
    if (prk::overlap(A, order * order * 8, B, order * order * 8))
        return prk::record_error(PRK_ERR_ARG, "transpose: A and B overlap");
    const int vec = (reinterpret_cast<uintptr_t>(A) & 15u) == 0 && order % 2 == 0;
    const dim3 grid(static_cast<unsigned>(tiles), static_cast<unsigned>(tiles));
    prk::k_transpose<<<grid, prk::TR_THREADS, 0, static_cast<cudaStream_t>(stream)>>>(order, A, B, vec);
    if (cudaError_t e = cudaGetLastError()) return prk::record_error(PRK_ERR_STATE, cudaGetErrorString(e));
    return PRK_OK;
}

}  // extern "C"
