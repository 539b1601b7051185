"""The C ABI library and the host driver without a GPU: symbols, pure host functions, argument
checks (rejected before any CUDA call), and the CLI's reference-compatible argument errors."""
import ctypes as C
import subprocess
from pathlib import Path

import pytest

import kernels_gb300 as kg
from kernels_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]
CLI = ROOT / "kernels_gb300" / "_build" / "stencil-gb300"


def test_library_exports_every_header_symbol():
    lib = _lib.load()
    declared = _lib.header_symbols()
    assert len(declared) >= 10
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) <= set(_lib.SIGNATURES)


def test_version_and_pure_functions():
    lib = _lib.load()
    assert "sm_103a" in kg.version()
    assert lib.prk_gb300_bytes(16384, kg.FP64, 0) == 16384 * 16384 * 8
    assert lib.prk_gb300_bytes(16384, kg.FP32C, 0) == 16384 * 16384 * 4
    assert lib.prk_gb300_bytes(16384, kg.FP32C, 1) == 16384 * 16384 * 8
    assert lib.prk_gb300_bytes(0, kg.FP64, 0) == -1
    assert kg.flops(kg.STAR, 2, 16384) == 19 * 16380.0 ** 2
    assert kg.flops(kg.GRID, 5, 1000) == (2 * 121 + 1) * 990.0 ** 2


def test_route_split_covers_every_add_of_the_chain():
    """prk_gb300_route_split: for the stencils whose weights are not powers of two, the fixed-point
    and binary64 adds of one application per point are the chain's taps - 1 adds plus the add into
    out, in launches of one application and of several (one split for every depth above 1); most of
    each chain runs in fixed point. The power-of-two stencils, a radius outside 1..5 and a depth below
    1 are rejected."""
    for p, r in [(kg.STAR, 3), (kg.STAR, 4), (kg.STAR, 5), (kg.GRID, 2), (kg.GRID, 3), (kg.GRID, 4), (kg.GRID, 5)]:
        taps = 4 * r if p == kg.STAR else 4 * r * r + 2 * r
        one, many = kg.route_split(p, r, 1), kg.route_split(p, r, 8)
        for fixed, dp in (one, many):
            assert fixed + dp == taps, (p, r)
            assert taps // 2 <= fixed < taps and dp >= 2
        assert kg.route_split(p, r, 100) == many
    for p, r in [(kg.STAR, 1), (kg.STAR, 2), (kg.GRID, 1)]:
        assert kg.route_split(p, r) is None
    f, d = C.c_int(), C.c_int()
    assert _lib.load().prk_gb300_route_split(kg.STAR, 6, 1, C.byref(f), C.byref(d)) == -1
    assert _lib.load().prk_gb300_route_split(kg.STAR, 3, 0, C.byref(f), C.byref(d)) == -1


@pytest.mark.parametrize("args,code", [
    ((kg.STAR, 0, 100, kg.FP64), -1),     # radius < 1
    ((kg.STAR, 6, 100, kg.FP64), -1),     # radius > 5
    ((kg.GRID, 3, 6, kg.FP64), -1),       # 2R+1 > n
    ((kg.STAR, 2, 0, kg.FP64), -1),       # n < 1
    ((7, 2, 100, kg.FP64), -1),           # unknown pattern
    ((kg.STAR, 2, 100, 9), -1),           # unknown dtype
    ((kg.STAR, 2, 1 << 40, kg.FP64), -5),  # above the addressable maximum
])
def test_stencil_rejects_bad_arguments_without_launching(args, code):
    lib = _lib.load()
    rc = lib.prk_gb300_stencil(*args, C.c_void_p(0x1000), None, C.c_void_p(0x100000), None)
    assert rc == code
    assert lib.prk_gb300_last_error()


def test_null_and_overlapping_buffers_rejected():
    lib = _lib.load()
    assert lib.prk_gb300_stencil(kg.STAR, 2, 100, kg.FP64, None, None, C.c_void_p(0x100000), None) == -1
    # in and out overlap
    assert lib.prk_gb300_stencil(kg.STAR, 2, 100, kg.FP64, C.c_void_p(0x1000), None, C.c_void_p(0x1008), None) == -1
    assert b"overlap" in lib.prk_gb300_last_error()
    assert lib.prk_gb300_run(kg.STAR, 2, 100, kg.FP64, 0, C.c_void_p(0x1000), C.c_void_p(0x200000),
                             C.c_void_p(0x400000), 0, None, None, None) == -1


def _cli(*args):
    return subprocess.run([str(CLI), *map(str, args)], capture_output=True, text=True, timeout=60)


@pytest.mark.parametrize("args,msg", [
    ((), "Usage: <# iterations> <array dimension> [<tile_size> <star/grid> <radius>]"),
    ((0, 100), "ERROR: iterations must be >= 1"),
    ((10, 0), "ERROR: grid dimension must be positive"),
    ((10, 4, 32, "grid", 2), "ERROR: Stencil radius negative or too large"),
    ((10, 100, 32, "star", 0), "ERROR: Stencil radius negative or too large"),
    ((10, 100, 32, "star", 2, "--unfused", "--whole"), "ERROR: --tuned and --whole are fused forms"),
])
def test_cli_argument_errors_match_reference(args, msg):
    assert CLI.exists(), "stencil-gb300 was not built"
    res = _cli(*args)
    assert res.returncode == 1
    assert res.stdout.splitlines()[0] == "Parallel Research Kernels"
    assert msg in res.stdout
