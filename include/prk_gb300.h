/*
 * prk_gb300.h - C ABI of the GB300 (sm_103a) PRK 2D stencil library, libprk_gb300.so.
 *
 * The library replaces the stencil hot path of the Parallel Research Kernels' C++11 drivers
 * (paths below are within the ParRes/Kernels project):
 *
 *   Cxx11/stencil_openmp.hpp:1       void starR/gridR(const int n, const int t, const double* in, double* out)
 *   Cxx11/stencil_cuda.hpp:1         __global__ void starR/gridR(const int n, const prk_float* in, prk_float* out)
 *   Cxx11/stencil-openmp.cc:208-218  the in += 1.0 sweep after each application
 *   Cxx11/stencil-cuda.cu:76-84      __global__ void add(const int n, prk_float* in)
 *   Cxx11/stencil-openmp.cc:230-239  L1 norm of out over the interior, divided by (n-2R)^2
 *   Cxx11/stencil-openmp.cc:182-223  the driver's init and timed iteration loop
 *
 * Conventions shared by every entry point:
 *   - Arrays are row-major n x n, element (i,j) at i*n+j, indices 64-bit (n is not capped at
 *     46340 as prk::get_max_matrix_size() caps it, Cxx11/prk_util.h:373-377).
 *   - Device pointers are owned by the caller (cudaMalloc alignment, 256 B, gives the fast path;
 *     any 8-byte-aligned pointer works). The library allocates only where an entry point says so.
 *   - dtype PRK_FP64: in, in_next, out are double[n*n].
 *     dtype PRK_FP32C: in, in_next are float[n*n]; out is float[2*n*n], interleaved (hi, lo) pairs
 *     whose unevaluated sum hi+lo is the value (a compensated two-float accumulator).
 *   - stream is a cudaStream_t passed as void* (NULL = the legacy default stream). Calls are
 *     stream-ordered and asynchronous unless stated otherwise. Calls on one stream from one host
 *     thread at a time.
 *   - Return value: 0 on success; a negative PRK_ERR_* code for a rejected call (nothing was
 *     launched); a positive cudaError_t value when the CUDA runtime failed. The library never
 *     aborts the process; prk_gb300_last_error() gives the message of the calling thread's last
 *     failure.
 */
#ifndef PRK_GB300_H
#define PRK_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PRK_STAR 0
#define PRK_GRID 1

#define PRK_FP64 0
#define PRK_FP32C 1

#define PRK_OK 0
#define PRK_ERR_ARG (-1)     /* bad pattern, radius, n, dtype, iteration count or pointer */
#define PRK_ERR_NOMEM (-2)   /* a library-owned allocation failed */
#define PRK_ERR_STATE (-3)   /* call out of order (e.g. batch not prepared) */
#define PRK_ERR_TIMEOUT (-4) /* a bounded device-side wait gave up (batched queue) */
#define PRK_ERR_LIMIT (-5)   /* a size is above a documented fixed maximum */

/* Flags for prk_gb300_run(). */
#define PRK_RUN_GRAPH 1   /* capture the timed iteration loop in a CUDA graph and replay it */
#define PRK_RUN_UNFUSED 2 /* reference structure: stencil kernel, then a separate in += 1 pass */
/* Temporal depth d in {1, 2, 4, 8}: each launch applies d consecutive applications to a tile held
 * in shared memory (the fused form on the tile kernels; depth 1 for PRK_RUN_UNFUSED and the generic
 * kernels). */
#define PRK_RUN_DEPTH(d) ((d) << 8)
/* Tall tiles: 64 rows per TMA tile (8 rows per thread) instead of 32 (4 per thread). */
#define PRK_RUN_TALL 8
/* All timed applications in one launch: every tile carries iterations 1..K in shared memory (in
 * evolves pointwise, so a tile needs only its own rows and the R-row halo of the initial in). The
 * results are those of K single applications. The fused form only, on the tile kernels (as
 * prk_gb300_stencil_steps); overrides PRK_RUN_DEPTH and the tuned depth. */
#define PRK_RUN_WHOLE 16

/* One application of the stencil (replaces starR/gridR, stencil_openmp.hpp:1, stencil_cuda.hpp:1):
 *   out[i*n+j] += sum over taps of w * in[(i+dr)*n + (j+dc)]   for R <= i,j < n-R,
 * evaluated in the generator's tap order (generate-cxx-stencil.py:15-38).
 * With in_next != NULL it also writes in_next = in + 1 over all n*n points (the fused form of the
 * sweep at stencil-openmp.cc:208-218); in_next must not overlap in or out.
 * With in_next == NULL it is exactly the reference operator: out is updated, in is untouched.
 * PRK_FP64 results are bit-identical to the reference's strict-order binary64 evaluation. */
int prk_gb300_stencil(int pattern, int radius, int64_t n, int dtype, const void* in, void* in_next, void* out,
                      void* stream);

/* `steps` consecutive fused applications in one launch (temporal blocking), steps in {1, 2, 4, 8}:
 * out += S(in) + S(in+1) + ... + S(in+steps-1) with out rounded after every application exactly as
 * `steps` single applications round it, and in_next = in + steps (each +1 rounded in turn). Every
 * application reads the in values and applies every tap; only the HBM round trips between them are
 * saved. in is not modified. The TMA tile kernels take 16-byte-aligned buffers with n a multiple of
 * 2 (PRK_FP64) or 4 (PRK_FP32C); other shapes run on the plain-staged tile kernels and need buffers
 * aligned to their element size (8 bytes for out and PRK_FP64 in, 4 for PRK_FP32C in), else
 * PRK_ERR_ARG. No counterpart in the reference, whose loop always makes the round trip
 * (Cxx11/stencil-openmp.cc:197-219). */
int prk_gb300_stencil_steps(int pattern, int radius, int64_t n, int dtype, int steps, const void* in, void* in_next,
                            void* out, void* stream);

/* in += 1 over all n*n points in place (stencil-openmp.cc:208-218, stencil-cuda.cu:76-84). */
int prk_gb300_add(int64_t n, int dtype, void* in, void* stream);

/* The drivers' initialisation (stencil-openmp.cc:184-195): in(i,j) = i+j, out = 0. */
int prk_gb300_init(int64_t n, int dtype, void* in, void* out, void* stream);

/* L1 norm of out over the interior divided by (n-2R)^2 (stencil-openmp.cc:230-239), reduced on
 * the device in binary64 with a fixed order. Synchronous: waits for the stream and writes *norm.
 * Uses a library-owned device scratch buffer, allocated once per device on first use. */
int prk_gb300_norm(int radius, int64_t n, int dtype, const void* out, double* norm, void* stream);

/* A whole PRK run on caller-owned device buffers (stencil-openmp.cc:197-223 / stencil-cuda.cu:211-222):
 * iterations+1 applications, each followed by the in += 1 sweep; iteration 0 is the untimed warm-up
 * and *elapsed_s receives the time of iterations 1..K measured with CUDA events on `stream`.
 * The fused form ping-pongs between in_a (holding the initial in) and in_b; *final_in is set to 0
 * or 1 for the buffer that holds the final in. With PRK_RUN_UNFUSED, in_b may be NULL and in_a is
 * updated in place. Synchronous. */
int prk_gb300_run(int pattern, int radius, int64_t n, int dtype, int iterations, void* in_a, void* in_b, void* out,
                  int flags, double* elapsed_s, int* final_in, void* stream);

/* A whole PRK run from host memory, the way Cxx11/stencil-cuda.cu drives it (:193-226): copies
 * h_in and h_out to the device, runs iterations+1 fused applications, copies out (and the final in,
 * when h_in_final != NULL) back, and computes the norm. The grid goes in bands of rows: each band's
 * copies in, its one launch carrying all iterations+1 applications (TMA tiles, or plain-staged
 * tiles for an n the TMA tiles cannot take), and its copies back overlap those of the other bands.
 * With PRK_CFG_KERNEL 1 (generic kernels only) it copies in, runs with the autotuner's choice
 * (PRK_RUN_TUNED) and copies back; with 2 (TMA required) an n the TMA tiles cannot take is
 * PRK_ERR_ARG. Its device
 * buffers and streams are allocated on first use and kept for later calls (the buffers grown when
 * a larger grid comes); prk_gb300_release frees them. Calls are serialised process-wide.
 * *elapsed_s (optional) is the whole call's wall time including the copies; *kernel_s (optional)
 * the event time of the evaluation: the span of the band launches, or iterations 1..K. Host
 * buffers may be pageable or pinned (pinned ones let the copies overlap). */
int prk_gb300_run_host(int pattern, int radius, int64_t n, int dtype, int iterations, const void* h_in, void* h_out,
                       void* h_in_final, double* norm, double* elapsed_s, double* kernel_s);

/* ---- One grid split across ranks in row slabs ---------------------------------------------
 * The reference splits a grid into blocks, one per MPI rank, exchanges an R-wide halo with the
 * neighbouring ranks before every application, applies the stencil to its block and adds one to its
 * in, then sums the ranks' norms (MPI1/Stencil/stencil.c:199-268 block split, :338-404 exchange,
 * :406-420 stencil and in += 1, :425-436 reductions). Here a rank owns the grid rows [row_begin,
 * row_end) (whole rows, so every halo is contiguous rows of the neighbours' slabs) and its buffers
 * hold its slab with the halo: grid rows [halo_begin, halo_end) with halo_begin = max(0,
 * row_begin - R) and halo_end = min(n, row_end + R), row stride n, element layout as for whole
 * grids. kernels_gb300.decomp does the split, the exchange and the reductions.
 *
 * prk_gb300_slab_run: `apps` (>= 1) fused applications in one launch. in holds the current in on
 * every row of the buffers (the halo rows as the neighbours sent them); in evolves pointwise, so an
 * R-row halo serves any number of applications. The call adds each application's stencil into out
 * on the slab's interior points (in the generator's order, as prk_gb300_stencil; FP64 bit-identical
 * to the whole grid's result) and writes in + apps into in_next on the rows [row_begin, row_end);
 * in_next's halo rows are not written (the next exchange fills them). Buffers 16-byte aligned with
 * n a multiple of 2 (FP64) or 4 (FP32C) take the TMA tiles, others the plain-staged tiles.
 * Stream-ordered. */
int prk_gb300_slab_run(int pattern, int radius, int64_t n, int dtype, int apps, int64_t row_begin, int64_t row_end,
                       const void* in, void* in_next, void* out, void* stream);

/* The sum of |out| over the slab's interior points (not divided by (n-2R)^2: the ranks' sums are
 * added first, as MPI1/Stencil/stencil.c:425-436 reduces them). out is a slab buffer as above.
 * Synchronous. */
int prk_gb300_slab_norm(int radius, int64_t n, int dtype, int64_t row_begin, int64_t row_end, const void* out,
                        double* l1_sum, void* stream);

/* Capacity of the fixed scratch behind prk_gb300_norm_noalloc: partial sums, 8 KiB per device. */
#define PRK_NOALLOC_NORM_PARTIALS 1024

/* The L1 norm of prk_gb300_norm, for callers that cannot let the library allocate device memory
 * (a framework whose caching allocator owns the device's memory, a service on a fixed memory
 * budget, a loop that cannot afford cudaMalloc's implicit device synchronisation). No counterpart
 * in the reference: the reference computes its norm on the host after copying out back.
 * - Allocates nothing: no cudaMalloc, cudaFree or allocating library call. Its scratch is a fixed
 *   array of PRK_NOALLOC_NORM_PARTIALS doubles inside the library's device image, held by every
 *   device that loads the library until the process exits; a reduction that would need more
 *   partial sums is rejected with PRK_ERR_LIMIT (with the norm's fixed block count, none does).
 * - norm_dev is caller-owned DEVICE memory for one double; the result is the same value
 *   prk_gb300_norm returns. Stream-ordered and asynchronous: read *norm_dev after the stream.
 * - The first call on each device looks up the scratch's device address (cudaGetSymbolAddress)
 *   with that device current, and keeps it for the CUDA context it belongs to; the first call in a
 *   new context on that device (e.g. after cudaDeviceReset) looks it up again. Make those first
 *   calls before any stream capture.
 * - Every call shares the scratch, which keeps the last call's contents (nothing in it needs to
 *   start at zero). Calls that overlap on the GPU, e.g. on two streams, race on it. */
int prk_gb300_norm_noalloc(int radius, int64_t n, int dtype, const void* out, double* norm_dev, void* stream);

/* Process-wide settings. PRK_CFG_KERNEL selects the stencil kernel family: 0 = automatic (for the
 * fused form, the TMA tile kernels on 16-byte-aligned buffers with n a multiple of 2 (FP64) or 4
 * (FP32C) and the plain-staged tile kernels on other shapes; the generic kernels for the form
 * without in_next), 1 = generic kernels only, 2 = TMA kernels required (calls that are not
 * eligible fail with PRK_ERR_ARG). Returns the previous value, or a negative error. Callable from
 * any thread; it governs the calls that start after it returns. */
#define PRK_CFG_KERNEL 1
int prk_gb300_config(int key, int value);

/* Reads and clears the device status word of the current device: PRK_OK, or PRK_ERR_TIMEOUT when a
 * kernel's bounded wait on its tile loads gave up since the last check. Synchronises the device.
 * prk_gb300_run checks it after every run. */
int prk_gb300_status(void);

/* ---- Autotuner ----------------------------------------------------------------------------
 * Picks, per (pattern, radius, n, dtype), the kernel family, tile shape, thread coarsening and
 * temporal depth by timing the candidates on scratch buffers of the same shape (n capped at 8192;
 * larger grids share the 8192 result, their per-point cost being the same). Results are kept in
 * memory and in a cache file, one JSON object per line: $PRK_GB300_TUNE_CACHE, else
 * $HOME/.cache/prk_gb300/tune.jsonl. No counterpart in the reference (whose tile size is a CLI
 * argument, Cxx11/stencil-openmp.cc:111-116). */
typedef struct {
    int depth;                      /* applications per launch: 1, 2, 4 or 8; 0: every timed
                                       application in one launch (PRK_RUN_WHOLE) */
    int kernel;                     /* 1 = generic kernels, 2 = TMA tile kernels, 3 = batched kernel,
                                       4 = plain-staged tile kernels (shapes TMA cannot take) */
    int tile_rows;                  /* tile shape (rows x columns) of the chosen kernel */
    int tile_cols;
    int cols_per_thread;            /* thread coarsening: adjacent columns each thread owns */
    double seconds_per_application; /* measured on the scratch grid */
    int from_cache;                 /* 1 when the result came from the cache */
} prk_gb300_tuning;

#define PRK_TUNE_BATCH 1 /* tune the batched kernel for a grid of this n */
#define PRK_TUNE_FORCE 2 /* measure again even when cached */
int prk_gb300_tune(int pattern, int radius, int64_t n, int dtype, int flags, prk_gb300_tuning* result);

/* Flag for prk_gb300_run: take the temporal depth and kernel family from prk_gb300_tune. */
#define PRK_RUN_TUNED 4

/* ---- Batched grids ------------------------------------------------------------------------
 * Many independent PRK grids of uneven n, mixed radius and pattern, advanced together: every launch
 * is one persistent kernel over the tiles of all grids, which CTAs take from a device work queue.
 * No counterpart in the reference, where each grid is a separate run of the driver
 * (Cxx11/stencil-openmp.cc). One grid's buffers follow the prk_gb300_run conventions: in_a holds
 * the initial in, in_b the second in buffer, out the accumulator; any n >= 2R+1 and alignment. */
typedef struct {
    int pattern;
    int radius;
    int64_t n;
    void* in_a;
    void* in_b;
    void* out;
} prk_gb300_grid;

typedef struct prk_gb300_batch prk_gb300_batch;

/* Builds a batch over `count` grids of one dtype (the descriptors are copied; the buffers stay
 * caller-owned). flags: PRK_RUN_DEPTH(d) fixes the temporal depth of every grid; PRK_RUN_WHOLE
 * runs every grid's timed applications in one launch; PRK_BATCH_TUNED takes each grid's depth
 * (0 for the whole run) from the autotuner (prk_gb300_tune), grouping grids by depth. Allocates
 * the batch's device tables. */
#define PRK_BATCH_TUNED 0x10000
int prk_gb300_batch_create(const prk_gb300_grid* grids, int count, int dtype, int flags, prk_gb300_batch** batch);

/* iterations+1 fused applications of every grid of the batch (application 0 untimed, as in
 * prk_gb300_run). *elapsed_s gets the event time of applications 1..K. With PRK_RUN_GRAPH the
 * timed launches are captured once into a CUDA graph (per iteration count) and replayed.
 * Synchronous. */
int prk_gb300_batch_run(prk_gb300_batch* batch, int iterations, int flags, double* elapsed_s, void* stream);

/* 0 or 1: which of grid `index`'s buffers (in_a, in_b) holds its final in after the last run;
 * negative for a bad index. */
int prk_gb300_batch_final_in(const prk_gb300_batch* batch, int index);

/* The interior L1 norm / (n-2R)^2 of every grid's out, into norms[count]. Synchronous. */
int prk_gb300_batch_norms(prk_gb300_batch* batch, double* norms, void* stream);

/* Launches per run of `iterations` (after the warm-up launch), for the benchmark's launch count. */
int prk_gb300_batch_launches(const prk_gb300_batch* batch, int iterations);

int prk_gb300_batch_destroy(prk_gb300_batch* batch);

/* Failure-path self-test: runs a kernel whose bounded mbarrier wait runs out by construction (a
 * barrier nobody arrives on, a short poll limit) and returns what prk_gb300_status reports then:
 * PRK_ERR_TIMEOUT when the timeout path works. The GPU stays usable; nothing faults or hangs. */
int prk_gb300_selftest_timeout(void);

/* Measures the current device's binary64 add throughput (adds per second) with a short kernel of
 * independent add chains on every SM. The strict-order FP64 stencils (weights that are not powers of
 * two) need one rounded binary64 add per tap, so this rate is their second ceiling beside HBM; the
 * benchmark reports both. Synchronous. No counterpart in the reference. */
int prk_gb300_probe_dadd(double* adds_per_second);

/* How the FP64 form of a stencil whose weights are not powers of two (star R=3..5, grid R=2..5) splits
 * the rounded adds of one application per interior point on whole-number tiles, in launches of
 * `depth` applications (1: one application per launch; more: temporal blocking or a whole run, which
 * move a larger share to the integer pipes): *fixed_adds run in exact fixed point on the integer
 * pipes, *binary64_adds on the binary64 pipe (the rest of the reference's chain and the add into
 * out). Both give the reference's bits; the split sets the kernel's two arithmetic ceilings.
 * PRK_ERR_ARG for the power-of-two stencils or a depth below 1. No counterpart in the reference. */
int prk_gb300_route_split(int pattern, int radius, int depth, int* fixed_adds, int* binary64_adds);

/* Frees the device buffers and streams prk_gb300_run_host keeps on the current device. */
int prk_gb300_release(void);

/* ---- Neighbouring PRK kernels on the same bandwidth roofline ---------------------------------
 * One application per call on caller-owned device memory, stream-ordered, binary64 with every
 * product and sum rounded on its own in the reference's order. */

/* The STREAM triad A[i] += B[i] + scalar * C[i] for i < length (replaces the nstream kernel of
 * Cxx11/nstream-cuda.cu:68-76 and its launch at :164-176). A must not overlap B or C. */
int prk_gb300_nstream(int64_t length, double scalar, double* A, const double* B, const double* C, void* stream);

/* B += A^T, then A += 1, for order x order row-major matrices (replaces transposeNoBankConflict<true>
 * of Cxx11/transpose-cuda.cu:63-86 and its launch at :223-246; any order up to 65535 * 64, not only
 * multiples of the tile). A and B must not overlap. */
int prk_gb300_transpose(int64_t order, double* A, double* B, void* stream);

/* Bytes one buffer of the given role needs: role 0 = in / in_next, role 1 = out. */
int64_t prk_gb300_bytes(int64_t n, int dtype, int role);

/* PRK's flop count for one application, (2*stencil_size+1)*(n-2R)^2 (stencil-openmp.cc:253-255). */
double prk_gb300_flops(int pattern, int radius, int64_t n);

/* Message of the calling thread's last failed call ("" when none). */
const char* prk_gb300_last_error(void);

/* Library version string. */
const char* prk_gb300_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PRK_GB300_H */
