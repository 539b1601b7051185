"""The reference's own CUDA stencil on the GPU, as a comparator (test infrastructure only).

oracle/_ref/stencil_cuda.cubin is the device code of Cxx11/stencil-cuda.cu (with the generated
kernels of Cxx11/stencil_cuda.hpp), compiled for sm_103a by `make -C oracle ref-cuda` from the
reference sources where they lie; it is git-ignored and travels with the working tree. This module
loads it through the CUDA driver API (ctypes on libcuda) in the process's current context and
drives it the way stencil-cuda.cu:88-89,211-222 does:

  dimGrid(ceil(n/tile), ceil(n/tile)), dimBlock(tile, tile);
  for iter in 0..K: stencil<<<>>>(n, in, out); add<<<>>>(n, in); cudaDeviceSynchronize()

with iteration 0 outside the timed region. Only the tests use it.
"""
from __future__ import annotations

import ctypes as C
import time
from pathlib import Path

CUBIN = Path(__file__).resolve().parent / "_ref" / "stencil_cuda.cubin"

_state: dict = {}


def available() -> bool:
    return CUBIN.exists()


def _cu():
    if "lib" not in _state:
        lib = C.CDLL("libcuda.so.1")
        vp = C.c_void_p
        lib.cuModuleLoad.argtypes = [C.POINTER(vp), C.c_char_p]
        lib.cuModuleGetFunction.argtypes = [C.POINTER(vp), vp, C.c_char_p]
        lib.cuLaunchKernel.argtypes = [vp, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, vp,
                                       C.POINTER(vp), C.POINTER(vp)]
        lib.cuCtxSynchronize.argtypes = []
        _state["lib"] = lib
    return _state["lib"]


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what}: CUDA driver error {rc}")


def _function(name: str):
    """A kernel of the module by its C++ name: star1..5, grid1..5 take (const int, const double*,
    double*), add takes (const int, double*)."""
    lib = _cu()
    if "mod" not in _state:
        mod = C.c_void_p()
        _check(lib.cuModuleLoad(C.byref(mod), str(CUBIN).encode()), "cuModuleLoad")
        _state["mod"] = mod
    key = "fn_" + name
    if key not in _state:
        mangled = f"_Z{len(name)}{name}iPKdPd" if name != "add" else "_Z3addiPd"
        fn = C.c_void_p()
        _check(lib.cuModuleGetFunction(C.byref(fn), _state["mod"], mangled.encode()), f"cuModuleGetFunction {mangled}")
        _state[key] = fn
    return _state[key]


def _launch(fn, grid: int, tile: int, args) -> None:
    holders = [C.c_int(args[0])] + [C.c_void_p(a) for a in args[1:]]
    params = (C.c_void_p * len(holders))(*[C.cast(C.pointer(h), C.c_void_p) for h in holders])
    _check(_cu().cuLaunchKernel(fn, grid, grid, 1, tile, tile, 1, 0, None, params, None), "cuLaunchKernel")


def run(pattern: str, radius: int, n: int, iterations: int, d_in: int, d_out: int, tile: int = 32) -> float:
    """iterations+1 applications on device buffers (in = d_in, out = d_out, both n*n float64, set by
    the caller); returns the wall time of iterations 1..K as stencil-cuda.cu measures it."""
    tile = max(1, min(tile, n))
    grid = (n + tile - 1) // tile
    stencil = _function(f"{pattern}{radius}")
    add = _function("add")
    lib = _cu()
    t0 = 0.0
    for it in range(iterations + 1):
        if it == 1:
            t0 = time.perf_counter()
        _launch(stencil, grid, tile, (n, d_in, d_out))
        _launch(add, grid, tile, (n, d_in))
        _check(lib.cuCtxSynchronize(), "cuCtxSynchronize")
    return time.perf_counter() - t0
