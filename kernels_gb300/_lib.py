"""ctypes binding of libprk_gb300.so, the C ABI declared in include/prk_gb300.h.

The library is built in-tree (kernels_gb300/_build/) by kernels_gb300.build. Loading fails loudly
when it is missing: there is no CPU fallback for the stencil path.
"""
from __future__ import annotations

import ctypes as C
import os
import re
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libprk_gb300.so"
HEADER = _PKG.parent / "include" / "prk_gb300.h"

_vp = C.c_void_p
_i64 = C.c_int64
_int = C.c_int
_dbl = C.c_double
_pd = C.POINTER(C.c_double)
_pi = C.POINTER(C.c_int)

# name -> (restype, argtypes); kept in the order of include/prk_gb300.h
SIGNATURES: dict[str, tuple] = {
    "prk_gb300_stencil": (_int, [_int, _int, _i64, _int, _vp, _vp, _vp, _vp]),
    "prk_gb300_stencil_steps": (_int, [_int, _int, _i64, _int, _int, _vp, _vp, _vp, _vp]),
    "prk_gb300_add": (_int, [_i64, _int, _vp, _vp]),
    "prk_gb300_init": (_int, [_i64, _int, _vp, _vp, _vp]),
    "prk_gb300_norm": (_int, [_int, _i64, _int, _vp, _pd, _vp]),
    "prk_gb300_slab_run": (_int, [_int, _int, _i64, _int, _int, _i64, _i64, _vp, _vp, _vp, _vp]),
    "prk_gb300_slab_norm": (_int, [_int, _i64, _int, _i64, _i64, _vp, _pd, _vp]),
    "prk_gb300_norm_noalloc": (_int, [_int, _i64, _int, _vp, _vp, _vp]),
    "prk_gb300_run": (_int, [_int, _int, _i64, _int, _int, _vp, _vp, _vp, _int, _pd, _pi, _vp]),
    "prk_gb300_run_host": (_int, [_int, _int, _i64, _int, _int, _vp, _vp, _vp, _pd, _pd, _pd]),
    "prk_gb300_config": (_int, [_int, _int]),
    "prk_gb300_status": (_int, []),
    "prk_gb300_selftest_timeout": (_int, []),
    "prk_gb300_tune": (_int, [_int, _int, _i64, _int, _int, C.c_void_p]),
    "prk_gb300_batch_create": (_int, [C.c_void_p, _int, _int, _int, C.c_void_p]),
    "prk_gb300_batch_run": (_int, [_vp, _int, _int, _pd, _vp]),
    "prk_gb300_batch_final_in": (_int, [_vp, _int]),
    "prk_gb300_batch_norms": (_int, [_vp, _vp, _vp]),
    "prk_gb300_batch_launches": (_int, [_vp, _int]),
    "prk_gb300_batch_destroy": (_int, [_vp]),
    "prk_gb300_probe_dadd": (_int, [_pd]),
    "prk_gb300_route_split": (_int, [_int, _int, _int, _pi, _pi]),
    "prk_gb300_release": (_int, []),
    "prk_gb300_nstream": (_int, [_i64, _dbl, _vp, _vp, _vp, _vp]),
    "prk_gb300_transpose": (_int, [_i64, _vp, _vp, _vp]),
    "prk_gb300_bytes": (_i64, [_i64, _int, _int]),
    "prk_gb300_flops": (_dbl, [_int, _int, _i64]),
    "prk_gb300_last_error": (C.c_char_p, []),
    "prk_gb300_version": (C.c_char_p, []),
}

class Tuning(C.Structure):
    """prk_gb300_tuning (include/prk_gb300.h)."""
    _fields_ = [("depth", C.c_int), ("kernel", C.c_int), ("tile_rows", C.c_int), ("tile_cols", C.c_int),
                ("cols_per_thread", C.c_int), ("seconds_per_application", C.c_double), ("from_cache", C.c_int)]


class Grid(C.Structure):
    """prk_gb300_grid (include/prk_gb300.h)."""
    _fields_ = [("pattern", C.c_int), ("radius", C.c_int), ("n", C.c_int64), ("in_a", C.c_void_p),
                ("in_b", C.c_void_p), ("out", C.c_void_p)]


_lib: C.CDLL | None = None


def header_symbols() -> list[str]:
    """Every function the public header declares (parsed from include/*.h)."""
    names: list[str] = []
    for h in sorted((HEADER.parent).glob("*.h")):
        text = h.read_text()
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(prk_gb300_[a-z0-9_]+)\s*\(", text, re.M)
    return names


def load() -> C.CDLL:
    """Load the library once and attach the ctypes signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = Path(os.environ.get("PRK_GB300_LIB", LIB_PATH))
    if not path.exists():
        raise ImportError(
            f"{path} is missing: build the CUDA library first (python -m kernels_gb300.build). "
            "The stencil path has no CPU fallback.")
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class PrkError(RuntimeError):
    """A failed library call: `code` is the return value (negative PRK_ERR_*, positive cudaError_t)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"prk_gb300 error {code}: {message}")
        self.code = code


def check(rc: int) -> None:
    if rc != 0:
        raise PrkError(rc, load().prk_gb300_last_error().decode())
