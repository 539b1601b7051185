"""prk_gb300_norm_noalloc: the allocation-free norm, for callers that cannot let a library call
cudaMalloc (a framework whose own allocator owns the device memory, a fixed memory budget, a loop
that must not synchronise the device). Its scratch is a fixed array in the library's device image,
so the test checks that it returns what prk_gb300_norm returns, on consecutive calls that share
that scratch, for both storage forms. Collected last so that a stop at the first failure has
already run every other test; it sets up everything it needs and also passes on its own.
"""
import ctypes as C

import numpy as np
import pytest

import kernels_gb300 as kg
from kernels_gb300 import _lib

pytestmark = pytest.mark.gpu

REL_TOL = 1e-13  # the tolerance the other norm checks use


def norm_noalloc(torch, radius, out, dtype):
    lib = _lib.load()
    res = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    rc = lib.prk_gb300_norm_noalloc(radius, int(out.shape[0]), dtype, out.data_ptr(), res.data_ptr(),
                                    torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.prk_gb300_last_error()
    torch.cuda.synchronize()
    return float(res.item())


@pytest.mark.parametrize("dtype", [kg.FP64, kg.FP32C])
def test_noalloc_norm_matches_allocating_norm(cuda, dtype):
    torch = cuda
    results = []
    for n, r, iters in ((1000, 2, 10), (517, 5, 3)):
        in_a, in_b, out = kg.alloc(n, dtype)
        kg.init(in_a, out)
        kg.run(kg.STAR, r, iters, in_a, in_b, out)
        want = kg.norm(r, out)
        first = norm_noalloc(torch, r, out, dtype)
        second = norm_noalloc(torch, r, out, dtype)  # same scratch, left over from the first call
        assert abs(first - want) <= REL_TOL * abs(want)
        assert abs(second - want) <= REL_TOL * abs(want)
        assert abs(want - 2.0 * (iters + 1)) <= 1e-8
        results.append(first)
    # a field with arbitrary values, after the calls above left the scratch full
    rng = np.random.default_rng(11)
    n = 777
    if dtype == kg.FP64:
        out = torch.from_numpy(rng.standard_normal((n, n)) * 1e3).cuda()
    else:
        out = torch.from_numpy(rng.standard_normal((n, n, 2)).astype(np.float32)).cuda()
        out[..., 1] *= 1e-8
    for _ in range(2):
        got = norm_noalloc(torch, 3, out, dtype)
        want = kg.norm(3, out)
        assert abs(got - want) <= REL_TOL * abs(want)


def test_noalloc_norm_rejects_bad_calls(cuda):
    lib = _lib.load()
    torch = cuda
    out = torch.zeros((64, 64), dtype=torch.float64, device="cuda")
    res = torch.zeros((1,), dtype=torch.float64, device="cuda")
    assert lib.prk_gb300_norm_noalloc(2, 1 << 40, kg.FP64, out.data_ptr(), res.data_ptr(), None) == -5
    assert b"maximum" in lib.prk_gb300_last_error()
    assert lib.prk_gb300_norm_noalloc(40, 64, kg.FP64, out.data_ptr(), res.data_ptr(), None) == -1
    assert lib.prk_gb300_norm_noalloc(2, 64, kg.FP64, out.data_ptr(), None, None) == -1
    assert lib.prk_gb300_norm_noalloc(2, 64, 7, out.data_ptr(), res.data_ptr(), None) == -1
