"""ctypes access to the CPU oracle (test infrastructure only).

liboracle.so  strict-rounding restatement of the reference stencil (parity oracle)
libprkcpu.so  the same source with the reference's -O3 -ffast-math -fopenmp flags (CPU baseline)

Only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module; the
shipped library never does. See prk_cpu_stencil.c for what each function restates.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF = HERE / "_ref"

STAR, GRID = 0, 1

_libs: dict[str, C.CDLL] = {}


def _load(name: str) -> C.CDLL:
    if name in _libs:
        return _libs[name]
    path = BUILD / name
    if not path.exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    lib = C.CDLL(str(path))
    vp, i64, i = C.c_void_p, C.c_int64, C.c_int
    lib.prk_oracle_weight.restype = C.c_double
    lib.prk_oracle_weight.argtypes = [i, i, i, i]
    lib.prk_oracle_taps.restype = i
    lib.prk_oracle_taps.argtypes = [i, i, vp, vp, vp]
    lib.prk_oracle_apply.restype = i
    lib.prk_oracle_apply.argtypes = [i, i, i64, i64, vp, vp]
    lib.prk_oracle_apply_rows.restype = i
    lib.prk_oracle_apply_rows.argtypes = [i, i, i64, i64, i64, i64, i64, vp, vp]
    lib.prk_oracle_add.restype = i
    lib.prk_oracle_add.argtypes = [i64, i64, vp]
    lib.prk_oracle_init.restype = i
    lib.prk_oracle_init.argtypes = [i64, i64, vp, vp]
    lib.prk_oracle_run.restype = i
    lib.prk_oracle_run.argtypes = [i, i, i64, i, i64, vp, vp, C.POINTER(C.c_double)]
    lib.prk_oracle_sample.restype = C.c_double
    lib.prk_oracle_sample.argtypes = [i, i, i64, i, i64, vp, vp]
    lib.prk_oracle_norm.restype = C.c_double
    lib.prk_oracle_norm.argtypes = [i, i64, vp]
    lib.prk_oracle_point.restype = C.c_double
    lib.prk_oracle_point.argtypes = [i, i, i64, i, i64, i64]
    lib.prk_oracle_flops.restype = C.c_double
    lib.prk_oracle_flops.argtypes = [i, i, i64]
    lib.prk_oracle_threads.restype = i
    lib.prk_oracle_threads.argtypes = []
    _libs[name] = lib
    return lib


def oracle() -> C.CDLL:
    return _load("liboracle.so")


def cpu_baseline() -> C.CDLL:
    return _load("libprkcpu.so")


def taps(pattern: int, radius: int) -> list[tuple[int, int, float]]:
    """(column offset, row offset, weight) in the generator's emission order."""
    dc = np.zeros(256, np.int32)
    dr = np.zeros(256, np.int32)
    w = np.zeros(256, np.float64)
    k = oracle().prk_oracle_taps(pattern, radius, dc.ctypes.data, dr.ctypes.data, w.ctypes.data)
    return [(int(dc[q]), int(dr[q]), float(w[q])) for q in range(k)]


def run(pattern: int, radius: int, n: int, iterations: int, tile: int = 32, in_=None, out=None):
    """A whole strict-order PRK run; returns (in, out) as float64 [n, n] arrays."""
    in_ = np.empty((n, n), np.float64) if in_ is None else in_
    out = np.empty((n, n), np.float64) if out is None else out
    el = C.c_double()
    rc = oracle().prk_oracle_run(pattern, radius, n, iterations, tile, in_.ctypes.data, out.ctypes.data, C.byref(el))
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    return in_, out


def apply(pattern: int, radius: int, in_: np.ndarray, out: np.ndarray, tile: int = 32) -> None:
    """One strict-order application out += S(in) on arbitrary float64 arrays (in place)."""
    assert in_.dtype == np.float64 and out.dtype == np.float64 and in_.flags.c_contiguous and out.flags.c_contiguous
    n = in_.shape[0]
    if oracle().prk_oracle_apply(pattern, radius, n, tile, in_.ctypes.data, out.ctypes.data) != 0:
        raise ValueError("oracle rejected the arguments")


def apply_rows(pattern: int, radius: int, n: int, first: int, row_begin: int, row_end: int, in_: np.ndarray,
               out: np.ndarray) -> None:
    """One strict-order application on a row slab (in place): in_ and out hold grid rows
    [first, first + in_.shape[0]) of an n x n grid; the interior points of rows [row_begin, row_end)
    are updated."""
    assert in_.dtype == np.float64 and out.dtype == np.float64 and in_.flags.c_contiguous and out.flags.c_contiguous
    assert in_.shape == out.shape and in_.shape[1] == n
    if oracle().prk_oracle_apply_rows(pattern, radius, n, first, in_.shape[0], row_begin, row_end, in_.ctypes.data,
                                      out.ctypes.data) != 0:
        raise ValueError("oracle rejected the slab arguments")


def norm(radius: int, out: np.ndarray) -> float:
    return float(oracle().prk_oracle_norm(radius, out.shape[0], out.ctypes.data))


def point(pattern: int, radius: int, n: int, applications: int, i: int, j: int) -> float:
    return float(oracle().prk_oracle_point(pattern, radius, n, applications, i, j))


def flops(pattern: int, radius: int, n: int) -> float:
    return float(oracle().prk_oracle_flops(pattern, radius, n))
