"""kernels_gb300: the PRK 2D stencil hot path on GB300 (sm_103a).

Host-side mirror of the reference operator interface over the C ABI (include/prk_gb300.h):

  star1..star5, grid1..grid5(n, t, in_, out)
      the reference operators' names and argument order (Cxx11/stencil_openmp.hpp:1,
      Cxx11/stencil_cuda.hpp:1): out += S(in) over the interior, in untouched. `t` (the CPU tile) is
      accepted and ignored.
  apply(pattern, radius, in_, out, in_next=None)
      one application; with in_next it also writes in_next = in + 1 (the fused sweep).
  add(in_)          in += 1 (Cxx11/stencil-openmp.cc:208-218)
  init(in_, out)    in = i+j, out = 0 (Cxx11/stencil-openmp.cc:184-195)
  norm(radius, out) interior L1 norm / (n-2R)^2 (Cxx11/stencil-openmp.cc:230-239)
  run(...)          a timed PRK run on device buffers (Cxx11/stencil-openmp.cc:197-223)
  run_host(...)     a PRK run from host arrays, copies included (Cxx11/stencil-cuda.cu:193-226)

Buffers are torch CUDA tensors (torch supplies device memory and streams only):
  FP64:  in_/in_next float64 [n, n]; out float64 [n, n]
  FP32C: in_/in_next float32 [n, n]; out float32 [n, n, 2] holding (hi, lo) pairs
Every call raises PrkError on failure, with the library's message; arguments the reference rejects
(radius outside 1..5, 2R+1 > n, iterations < 1) are rejected the same way.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from ._lib import PrkError, check, load

STAR, GRID = 0, 1
FP64, FP32C = 0, 1
RUN_GRAPH, RUN_UNFUSED, RUN_TUNED, RUN_TALL, RUN_WHOLE = 1, 2, 4, 8, 16

__all__ = ["STAR", "GRID", "FP64", "FP32C", "PrkError", "apply", "add", "init", "norm", "run", "run_host",
           "alloc", "apply_steps", "flops", "probe_dadd", "route_split", "slab_run", "slab_norm", "tune", "Batch", "pattern_of", "dtype_of", "version", "set_kernel", "status", "KERNEL_AUTO",
           "KERNEL_GENERIC", "KERNEL_TMA"] + \
          [f"{p}{r}" for p in ("star", "grid") for r in range(1, 6)]


def pattern_of(name: str) -> int:
    """The reference's rule (stencil-openmp.cc:124-128): "grid" selects grid, anything else star."""
    return GRID if name == "grid" else STAR


def dtype_of(t) -> int:
    import torch
    if t.dtype == torch.float64:
        return FP64
    if t.dtype == torch.float32:
        return FP32C
    raise PrkError(-1, f"unsupported tensor dtype {t.dtype}: use float64 (fp64) or float32 (fp32c)")


def _stream(stream) -> int | None:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return int(stream) if not hasattr(stream, "cuda_stream") else stream.cuda_stream


def _n_of(in_) -> int:
    if in_.dim() != 2 or in_.shape[0] != in_.shape[1] or not in_.is_contiguous():
        raise PrkError(-1, "in must be a contiguous square [n, n] tensor")
    return int(in_.shape[0])


def _check_out(out, n: int, dtype: int) -> None:
    import torch
    want = (n, n) if dtype == FP64 else (n, n, 2)
    wdt = torch.float64 if dtype == FP64 else torch.float32
    if tuple(out.shape) != want or out.dtype != wdt or not out.is_contiguous():
        raise PrkError(-1, f"out must be a contiguous {wdt} tensor of shape {want}")


KERNEL_AUTO, KERNEL_GENERIC, KERNEL_TMA = 0, 1, 2


def set_kernel(choice: int) -> int:
    """Select the stencil kernel family process-wide (PRK_CFG_KERNEL): KERNEL_AUTO, KERNEL_GENERIC
    or KERNEL_TMA. Returns the previous choice."""
    rc = load().prk_gb300_config(1, choice)
    if rc < 0:
        check(rc)
    return rc


def status() -> None:
    """Raise if a kernel's bounded wait gave up since the last check (synchronises the device)."""
    check(load().prk_gb300_status())


def version() -> str:
    return load().prk_gb300_version().decode()


def probe_dadd() -> float:
    """The current device's binary64 add throughput in adds per second (prk_gb300_probe_dadd): the
    ceiling of the strict-order FP64 stencils, which need one rounded add per tap."""
    res = C.c_double()
    check(load().prk_gb300_probe_dadd(C.byref(res)))
    return res.value


def route_split(pattern: int, radius: int, depth: int = 1) -> tuple[int, int] | None:
    """(fixed-point adds, binary64 adds) per interior point and application of the FP64 table route in
    launches of `depth` applications (prk_gb300_route_split), or None for the power-of-two stencils,
    which take the exact routes."""
    f, d = C.c_int(), C.c_int()
    rc = load().prk_gb300_route_split(pattern, radius, depth, C.byref(f), C.byref(d))
    return None if rc != 0 else (f.value, d.value)


def flops(pattern: int, radius: int, n: int) -> float:
    """PRK's flop count of one application, (2*stencil_size+1)*(n-2R)^2."""
    return float(load().prk_gb300_flops(pattern, radius, n))


def apply(pattern: int, radius: int, in_, out, in_next=None, stream=None) -> None:
    n = _n_of(in_)
    dt = dtype_of(in_)
    _check_out(out, n, dt)
    if in_next is not None and (in_next.shape != in_.shape or in_next.dtype != in_.dtype or not in_next.is_contiguous()):
        raise PrkError(-1, "in_next must match in")
    check(load().prk_gb300_stencil(pattern, radius, n, dt, in_.data_ptr(), None if in_next is None else in_next.data_ptr(),
                                   out.data_ptr(), _stream(stream)))


def apply_steps(pattern: int, radius: int, steps: int, in_, out, in_next, stream=None) -> None:
    """`steps` (1, 2, 4 or 8) fused applications in one launch: out accumulates every application,
    in_next = in + steps. Any n; buffers aligned to their element size (the TMA tiles where the
    layout allows them, the plain-staged tiles otherwise)."""
    n = _n_of(in_)
    dt = dtype_of(in_)
    _check_out(out, n, dt)
    if in_next.shape != in_.shape or in_next.dtype != in_.dtype or not in_next.is_contiguous():
        raise PrkError(-1, "in_next must match in")
    check(load().prk_gb300_stencil_steps(pattern, radius, n, dt, steps, in_.data_ptr(), in_next.data_ptr(),
                                         out.data_ptr(), _stream(stream)))


def _make_op(pattern: int, radius: int):
    def op(n: int, t: int, in_, out) -> None:
        if _n_of(in_) != n:
            raise PrkError(-1, f"n={n} does not match the tensor's {tuple(in_.shape)}")
        apply(pattern, radius, in_, out)
    op.__name__ = f"{'star' if pattern == STAR else 'grid'}{radius}"
    op.__doc__ = f"Reference operator {op.__name__}(n, t, in, out): out += S(in) over the interior."
    return op


star1, star2, star3, star4, star5 = (_make_op(STAR, r) for r in range(1, 6))
grid1, grid2, grid3, grid4, grid5 = (_make_op(GRID, r) for r in range(1, 6))


def add(in_, stream=None) -> None:
    check(load().prk_gb300_add(_n_of(in_), dtype_of(in_), in_.data_ptr(), _stream(stream)))


def init(in_, out, stream=None) -> None:
    n = _n_of(in_)
    dt = dtype_of(in_)
    _check_out(out, n, dt)
    check(load().prk_gb300_init(n, dt, in_.data_ptr(), out.data_ptr(), _stream(stream)))


def norm(radius: int, out, stream=None) -> float:
    import torch
    dt = FP64 if out.dtype == torch.float64 else FP32C
    n = int(out.shape[0])
    _check_out(out, n, dt)
    res = C.c_double()
    check(load().prk_gb300_norm(radius, n, dt, out.data_ptr(), C.byref(res), _stream(stream)))
    return res.value


@dataclass
class RunResult:
    elapsed_s: float   # event time of iterations 1..K
    final_in: object   # the tensor that holds the final `in`


def run(pattern: int, radius: int, iterations: int, in_a, in_b, out, graph: bool = False, unfused: bool = False,
        stream=None, depth: int = 1, tuned: bool = False, tall: bool = False, whole: bool = False) -> RunResult:
    n = _n_of(in_a)
    dt = dtype_of(in_a)
    _check_out(out, n, dt)
    el = C.c_double()
    fin = C.c_int()
    flags = (RUN_GRAPH if graph else 0) | (RUN_UNFUSED if unfused else 0) | (depth << 8) | (RUN_TUNED if tuned else 0) \
        | (RUN_TALL if tall else 0) | (RUN_WHOLE if whole else 0)
    check(load().prk_gb300_run(pattern, radius, n, dt, iterations, in_a.data_ptr(),
                               None if in_b is None else in_b.data_ptr(), out.data_ptr(), flags, C.byref(el),
                               C.byref(fin), _stream(stream)))
    return RunResult(el.value, in_a if fin.value == 0 else in_b)


def run_host(pattern: int, radius: int, iterations: int, h_in, h_out, h_in_final=None) -> dict:
    """A whole run from host arrays (numpy or CPU tensors); returns norm and timings."""
    def ptr(a):
        return a.ctypes.data if hasattr(a, "ctypes") else a.data_ptr()
    n = int(h_in.shape[0])
    import numpy as np
    dt = FP64 if h_in.dtype in (np.float64,) or str(h_in.dtype).endswith("float64") else FP32C
    nrm, el, ks = C.c_double(), C.c_double(), C.c_double()
    check(load().prk_gb300_run_host(pattern, radius, n, dt, iterations, ptr(h_in), ptr(h_out),
                                    None if h_in_final is None else ptr(h_in_final), C.byref(nrm), C.byref(el),
                                    C.byref(ks)))
    return {"norm": nrm.value, "elapsed_s": el.value, "kernel_s": ks.value}


def slab_run(pattern: int, radius: int, n: int, apps: int, row_begin: int, row_end: int, in_, in_next, out,
             stream=None) -> None:
    """`apps` fused applications on a row slab of an n x n grid (prk_gb300_slab_run): the tensors
    hold grid rows [max(0, row_begin - R), min(n, row_end + R)) with n columns (FP32C out: [.., n, 2]);
    out gains each application's stencil on the slab's interior points, in_next = in + apps on the
    rows [row_begin, row_end)."""
    dt = dtype_of(in_)
    lo, hi = max(0, row_begin - radius), min(n, row_end + radius)
    want = (hi - lo, n)
    for t in (in_, in_next):
        if tuple(t.shape) != want or dtype_of(t) != dt or not t.is_contiguous():
            raise PrkError(-1, f"slab in buffers must be contiguous {want} tensors of one dtype")
    if tuple(out.shape[:2]) != want or not out.is_contiguous():
        raise PrkError(-1, f"slab out must be a contiguous tensor of {want} points")
    check(load().prk_gb300_slab_run(pattern, radius, n, dt, apps, row_begin, row_end, in_.data_ptr(),
                                    in_next.data_ptr(), out.data_ptr(), _stream(stream)))


def slab_norm(radius: int, n: int, row_begin: int, row_end: int, out, stream=None) -> float:
    """Sum of |out| over a slab's interior points (prk_gb300_slab_norm), not yet divided by (n-2R)^2."""
    import torch
    dt = FP64 if out.dtype == torch.float64 else FP32C
    res = C.c_double()
    check(load().prk_gb300_slab_norm(radius, n, dt, row_begin, row_end, out.data_ptr(), C.byref(res), _stream(stream)))
    return res.value


def nstream(A, B, C_, scalar: float = 3.0, stream=None) -> None:
    """A += B + scalar * C on float64 device vectors of one length (prk_gb300_nstream)."""
    for t in (A, B, C_):
        if t.dtype != torch_float64() or not t.is_cuda or not t.is_contiguous() or t.numel() != A.numel():
            raise ValueError("nstream: A, B and C must be contiguous float64 CUDA tensors of one length")
    check(load().prk_gb300_nstream(A.numel(), scalar, A.data_ptr(), B.data_ptr(), C_.data_ptr(), _stream(stream)))


def transpose(A, B, stream=None) -> None:
    """B += A^T, then A += 1, on square float64 device matrices (prk_gb300_transpose)."""
    for t in (A, B):
        if t.dtype != torch_float64() or not t.is_cuda or not t.is_contiguous() or t.dim() != 2 \
                or t.shape[0] != t.shape[1] or t.shape != A.shape:
            raise ValueError("transpose: A and B must be square contiguous float64 CUDA tensors of one order")
    check(load().prk_gb300_transpose(A.shape[0], A.data_ptr(), B.data_ptr(), _stream(stream)))


def torch_float64():
    import torch
    return torch.float64


def tune(pattern: int, radius: int, n: int, dtype: int = FP64, batch: bool = False, force: bool = False) -> dict:
    """The autotuner's choice for (pattern, radius, n, dtype): kernel family, tile shape, thread
    coarsening and temporal depth (0: the whole run in one launch), measured on scratch buffers and
    cached (prk_gb300_tune)."""
    from ._lib import Tuning
    t = Tuning()
    check(load().prk_gb300_tune(pattern, radius, n, dtype, (1 if batch else 0) | (2 if force else 0), C.byref(t)))
    return {"depth": t.depth, "kernel": {1: "generic", 2: "tma", 3: "batched", 4: "plain"}.get(t.kernel, str(t.kernel)),
            "tile_rows": t.tile_rows, "tile_cols": t.tile_cols, "cols_per_thread": t.cols_per_thread,
            "seconds_per_application": t.seconds_per_application, "from_cache": bool(t.from_cache)}


class Batch:
    """Many independent grids advanced together by the batched persistent kernel
    (prk_gb300_batch_*). `grids` is a list of (pattern, radius, in_a, in_b, out) with device tensors;
    all of one dtype. depth fixes the temporal depth; whole=True runs every grid's timed applications
    in one launch; tuned=True takes the depth per grid from the tuner."""

    def __init__(self, grids, depth: int | None = None, tuned: bool = False, whole: bool = False):
        from ._lib import Grid
        if not grids:
            raise PrkError(-1, "a batch needs at least one grid")
        self._tensors = grids  # keep the buffers alive
        dt = dtype_of(grids[0][2])
        arr = (Grid * len(grids))()
        for k, (pattern, radius, in_a, in_b, out) in enumerate(grids):
            n = _n_of(in_a)
            if dtype_of(in_a) != dt:
                raise PrkError(-1, "all grids of a batch share one dtype")
            _check_out(out, n, dt)
            arr[k] = Grid(pattern, radius, n, in_a.data_ptr(), in_b.data_ptr(), out.data_ptr())
        flags = (depth or 0) << 8 | (0x10000 if tuned else 0) | (RUN_WHOLE if whole else 0)
        h = C.c_void_p()
        check(load().prk_gb300_batch_create(arr, len(grids), dt, flags, C.byref(h)))
        self._h = h
        self.dtype = dt

    def run(self, iterations: int, graph: bool = False, stream=None) -> float:
        el = C.c_double()
        check(load().prk_gb300_batch_run(self._h, iterations, RUN_GRAPH if graph else 0, C.byref(el), _stream(stream)))
        return el.value

    def final_in(self, k: int):
        which = load().prk_gb300_batch_final_in(self._h, k)
        if which < 0:
            raise PrkError(which, f"bad grid index {k}")
        return self._tensors[k][2] if which == 0 else self._tensors[k][3]

    def norms(self) -> list[float]:
        out = (C.c_double * len(self._tensors))()
        check(load().prk_gb300_batch_norms(self._h, out, _stream(None)))
        return list(out)

    def launches(self, iterations: int) -> int:
        return int(load().prk_gb300_batch_launches(self._h, iterations))

    def close(self) -> None:
        if getattr(self, "_h", None):
            load().prk_gb300_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def alloc(n: int, dtype: int = FP64, device="cuda", ping_pong: bool = True):
    """Device buffers for a run: (in_a, in_b or None, out), uninitialised."""
    import torch
    tdt = torch.float64 if dtype == FP64 else torch.float32
    in_a = torch.empty((n, n), dtype=tdt, device=device)
    in_b = torch.empty((n, n), dtype=tdt, device=device) if ping_pong else None
    out = torch.empty((n, n) if dtype == FP64 else (n, n, 2), dtype=tdt, device=device)
    return in_a, in_b, out
