// Internal launcher interface between the C ABI (capi.cu) and the kernel translation units.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "prk_stencil.cuh"

namespace prk {

// One stencil application as the C ABI describes it (prk_gb300_stencil). The buffers hold the whole
// n x n grid, or (nr > 0) a row slab of it: nr rows from grid row goff, row stride n
// (prk_gb300_slab_run).
struct StencilCall {
    int pattern;
    int R;
    int64_t n;
    int dtype;
    const void* in;
    void* in_next;  // may be null: stencil only, in untouched
    void* out;
    cudaStream_t stream;
    int64_t nr = 0;    // rows the buffers hold (0: n)
    int64_t goff = 0;  // grid row of the buffers' row 0
};

// Largest n the tile grids address (gridDim.y = ceil(n/16) <= 65535).
constexpr int64_t NMAX = 65535LL * 16;

// Bytes per point of one in buffer and of the out buffer.
inline int64_t in_elem_bytes(int dtype) { return dtype == FP64 ? 8 : 4; }
inline int64_t out_elem_bytes(int dtype) { return 8; }

// tile_host.cu: the TMA tile kernels, for the fused form on 16-byte-aligned buffers and rows.
// `steps` consecutive applications per launch (temporal depth 1, 2, 4 or 8). `status` is a device
// word; bit 0 is set if a bounded wait gave up.
bool tma_eligible(const StencilCall& c);
// Launches a kernel whose bounded mbarrier wait runs out by construction (tile_host.cu).
cudaError_t launch_wait_selftest(unsigned* status, cudaStream_t s);
bool tma_depth_ok(int steps);
// Tile heights the TMA kernels are built for (32 and 64 rows).
bool tma_rows_ok(int tile_rows);
cudaError_t launch_stencil_tma(const StencilCall& c, int steps, unsigned* status, int tile_rows = 32);
// All `depth` applications of a run in one launch over the tiles of buffer rows [row0, row0 + rows):
// reads `in` rows row0 - R .. row0 + rows + R - 1 (those the buffers hold; zero beyond) and the
// band's `out` rows, writes the band's in_next (in after `depth` updates) and out rows.
cudaError_t launch_stencil_tma_band(const StencilCall& c, int depth, int64_t row0, int64_t rows, unsigned* status);
// The same over buffer rows [row0, row0 + rows) with the compile-time depth `steps` (1, 2, 4 or 8).
cudaError_t launch_stencil_tma_rows(const StencilCall& c, int steps, int64_t row0, int64_t rows, unsigned* status);

// tile_plain_*.cu: the fused form on shapes the TMA kernels cannot take (any n, buffers aligned to
// their element size); the tile staged with plain loads, then evaluated as in the TMA kernels.
// `depth` applications in one launch (1 for one application per launch), over the tiles of buffer
// rows [row0, row0 + rows) (rows = 0: to the last row), reading `in` rows row0 - R .. row0 + rows +
// R - 1 as launch_stencil_tma_band does.
bool plain_eligible(const StencilCall& c);
cudaError_t launch_stencil_plain(const StencilCall& c, int depth, int64_t row0 = 0, int64_t rows = 0);

// kernels_generic.cu: any n, any 8-byte-aligned pointers.
cudaError_t launch_stencil_generic(const StencilCall& c);
cudaError_t launch_add(int64_t n, int dtype, void* in, cudaStream_t s);
cudaError_t launch_init(int64_t n, int dtype, void* in, void* out, cudaStream_t s);
// Writes the interior L1 norm / (n-2R)^2 to *result_dev; partial must hold NORM_BLOCKS doubles.
constexpr int NORM_BLOCKS = 1024;
cudaError_t launch_norm(int R, int64_t n, int dtype, const void* out, double* partial, double* result_dev,
                        cudaStream_t s);
// The sum of |out| over the interior columns R..n-R-1 of array rows [i_lo, i_hi) (row stride n),
// divided by `divisor`, to *result_dev; the same kernels and fixed order as launch_norm.
cudaError_t launch_norm_rows(int R, int64_t n, int dtype, const void* out, int64_t i_lo, int64_t i_hi, double divisor,
                             double* partial, double* result_dev, cudaStream_t s);

// Binary64 add throughput probe: `blocks` CTAs of 256 threads, 8 chains of `iters` adds each.
cudaError_t launch_dadd_probe(double* sink, int blocks, int iters, double step, cudaStream_t s);

// Unique id of the calling thread's current CUDA context (cuCtxGetId), 0 when there is none or the
// driver gives none (norm_noalloc.cu). Device addresses the library caches are kept with the id of
// the context they belong to: after cudaDeviceReset the device's context, and its memory, are new.
unsigned long long current_context_id();

// The table route's split of one application's adds per point for an FP64 stencil whose weights are
// not powers of two, in launches of `depth` applications (1, or more): adds done in fixed point on the
// integer pipes and rounded binary64 adds (the rest of the chain and the add into out). -1 for the
// other stencils (tile_host.cu).
int table_route_split(int pattern, int R, int depth, int* fixed_adds, int* binary64_adds);

// Records `msg` as the calling thread's prk_gb300_last_error() and returns `code` (capi.cu).
int record_error(int code, const char* msg);

}  // namespace prk
