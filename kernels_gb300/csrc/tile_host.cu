// Host side of the tile kernels: eligibility, tensor-map encoding and dispatch to the per-form
// instantiations of the TMA kernel (tile_*.cu) and of the plain-staging kernel (tile_plain_*.cu).
// cuTensorMapEncodeTiled is fetched from the driver at run time, so the library does not link
// libcuda.
#include <cudaTypedefs.h>

#include <mutex>

#include "tile_plain.cuh"

namespace prk {
namespace {

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;
cudaError_t g_encode_err = cudaSuccess;

cudaError_t encoder(PFN_cuTensorMapEncodeTiled_v12000* fn)
{
    std::call_once(g_encode_once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        g_encode_err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (g_encode_err == cudaSuccess && q != cudaDriverEntryPointSuccess) g_encode_err = cudaErrorNotSupported;
        g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    *fn = g_encode;
    return g_encode_err;
}

// A 2D map over a row-major array of nr rows of n elem_bytes elements, box (box_x, box_y), zero fill.
cudaError_t make_map(CUtensorMap* map, const void* base, int64_t n, int64_t nr, int elem_bytes, int box_x, int box_y)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
    if (cudaError_t e = encoder(&enc)) return e;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(n), static_cast<cuuint64_t>(nr)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(n) * elem_bytes};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(box_x), static_cast<cuuint32_t>(box_y)};
    const cuuint32_t estr[2] = {1, 1};
    const CUtensorMapDataType dt = elem_bytes == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const CUresult r = enc(map, dt, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace

namespace {

// A wait that must run out: the barrier expects one arrival that nobody makes. Every thread gives up
// after `limit` polls, and the CTA reports through the status word exactly as a stalled tile load
// would. No copy is in flight, so returning is safe.
__global__ void k_wait_timeout_selftest(unsigned* status, uint32_t limit)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&bar, 0, limit);
    __syncthreads();
    if (!ok && threadIdx.x == 0) atomicOr(status, 1u);
}

}  // namespace

cudaError_t launch_wait_selftest(unsigned* status, cudaStream_t s)
{
    k_wait_timeout_selftest<<<1, 64, 0, s>>>(status, 1000);
    return cudaGetLastError();
}

bool tma_eligible(const StencilCall& c)
{
    if (!c.in_next) return false;  // the reference-operator form (no in_next) uses the generic kernel
    const int vec = c.dtype == FP64 ? 2 : 4;
    auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
    return c.n % vec == 0 && c.n >= 8 && al16(c.in) && al16(c.in_next) && al16(c.out);
}

bool tma_depth_ok(int steps) { return steps == 1 || steps == 2 || steps == 4 || steps == 8; }

int table_route_split(int pattern, int R, int depth, int* fixed_adds, int* binary64_adds)
{
    int kf = -1, n = 0;
#define PRK_SPLIT(PP, RR)                                                                            \
    if (pattern == PP && R == RR) {                                                                  \
        if constexpr (tile::table_route<PP, RR, FP64>()) {                                            \
            kf = depth == 1 ? tile::fixed_taps<PP, RR, true>() : tile::fixed_taps<PP, RR, false>();    \
            n = tap_count(PP, RR);                                                                    \
        }                                                                                             \
    }
    PRK_SPLIT(STAR, 1) PRK_SPLIT(STAR, 2) PRK_SPLIT(STAR, 3) PRK_SPLIT(STAR, 4) PRK_SPLIT(STAR, 5)
    PRK_SPLIT(GRID, 1) PRK_SPLIT(GRID, 2) PRK_SPLIT(GRID, 3) PRK_SPLIT(GRID, 4) PRK_SPLIT(GRID, 5)
#undef PRK_SPLIT
    if (kf < 0) return -1;
    *fixed_adds = kf - 1;       // the fixed prefix starts from its first product
    *binary64_adds = n - kf + 1;  // the rest of the chain, and the add into out
    return 0;
}

bool tma_rows_ok(int tile_rows) { return tile_rows == tile::TH_DEFAULT || tile_rows == tile::TH_TALL; }

namespace {
cudaError_t launch_tma(const StencilCall& c, int steps, unsigned* status, int tile_rows, int depth, int64_t row0,
                       int64_t rows);
}  // namespace

cudaError_t launch_stencil_tma(const StencilCall& c, int steps, unsigned* status, int tile_rows)
{
    if (!tma_depth_ok(steps) || !tma_rows_ok(tile_rows)) return cudaErrorInvalidValue;
    return launch_tma(c, steps, status, tile_rows, 0, 0, 0);
}

bool plain_eligible(const StencilCall& c)
{
    if (!c.in_next || c.n > NMAX) return false;
    auto al = [](const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; };
    const uintptr_t e = c.dtype == FP64 ? 8 : 4;
    return al(c.in, e) && al(c.in_next, e) && al(c.out, 8);
}

cudaError_t launch_stencil_plain(const StencilCall& c, int depth, int64_t row0, int64_t rows)
{
    if (depth < 1 || !plain_eligible(c)) return cudaErrorInvalidValue;
    const plain::Args a{c.in, c.in_next, c.out, c.n, depth, c.stream, row0, rows, c.nr, c.goff};
    return c.dtype == FP64 ? plain::launch_fp64(c.pattern, c.R, a) : plain::launch_fp32c(c.pattern, c.R, a);
}

cudaError_t launch_stencil_tma_band(const StencilCall& c, int depth, int64_t row0, int64_t rows, unsigned* status)
{
    if (depth < 1 || row0 < 0 || rows < 1) return cudaErrorInvalidValue;
    return launch_tma(c, 0, status, tile::TH_DEFAULT, depth, row0, rows);
}

cudaError_t launch_stencil_tma_rows(const StencilCall& c, int steps, int64_t row0, int64_t rows, unsigned* status)
{
    if (!tma_depth_ok(steps) || row0 < 0 || rows < 1) return cudaErrorInvalidValue;
    return launch_tma(c, steps, status, tile::TH_DEFAULT, 0, row0, rows);
}

namespace {

cudaError_t launch_tma(const StencilCall& c, int steps, unsigned* status, int tile_rows, int depth, int64_t row0,
                       int64_t rows)
{
    tile::Launch L{};
    int ix, iy, ox, oy;
    tile::boxes(c.dtype, c.R, tile_rows, &ix, &iy, &ox, &oy);
    const int64_t nr = c.nr > 0 ? c.nr : c.n;
    if (cudaError_t e = make_map(&L.tm_in, c.in, c.n, nr, c.dtype == FP64 ? 8 : 4, ix, iy)) return e;
    if (cudaError_t e = make_map(&L.tm_out, c.out, c.n, nr, 8, ox, oy)) return e;
    L.nr = nr;
    L.goff = c.goff;
    L.n = c.n;
    L.in_next = c.in_next;
    L.out = c.out;
    L.status = status;
    L.stream = c.stream;
    L.depth = depth;
    L.row0 = row0;
    L.rows = rows;
    const bool tall = tile_rows == tile::TH_TALL;
    if (c.dtype == FP64) {
        if (c.pattern == STAR) return tall ? tile::launch_fp64_star_tall(c.R, steps, L) : tile::launch_fp64_star(c.R, steps, L);
        return tall ? tile::launch_fp64_grid_tall(c.R, steps, L) : tile::launch_fp64_grid(c.R, steps, L);
    }
    if (c.pattern == STAR) return tall ? tile::launch_fp32c_star_tall(c.R, steps, L) : tile::launch_fp32c_star(c.R, steps, L);
    return tall ? tile::launch_fp32c_grid_tall(c.R, steps, L) : tile::launch_fp32c_grid(c.R, steps, L);
}

}  // namespace

}  // namespace prk
