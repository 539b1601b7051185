"""Fused runs on shapes the TMA tiles cannot take: n not a multiple of the vector width, or buffers
that are not 16-byte aligned. These run on the plain-staged tile kernels (the tile loaded with plain
loads, then evaluated by the TMA kernels' code, with the same exact routes): the results must equal
the strict-order oracle bit for bit in FP64 and stay within the 1e-6 bound in FP32C, at every
temporal depth, for whole runs and for banded host-buffer runs, and match the generic kernels'."""
import numpy as np
import pytest

import kernels_gb300 as kg
from oracle import prk_oracle as po

pytestmark = pytest.mark.gpu

ALL = [(p, r) for p in (kg.STAR, kg.GRID) for r in range(1, 6)]


def bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def misaligned(torch, n, dtype):
    """in_a, in_b, out as views starting 8 bytes past a 16-byte boundary."""
    if dtype == kg.FP64:
        def one(shape):
            flat = torch.zeros(int(np.prod(shape)) + 1, dtype=torch.float64, device="cuda")
            return flat[1:].view(*shape)
        return one((n, n)), one((n, n)), one((n, n))
    def one32(shape):
        flat = torch.zeros(int(np.prod(shape)) + 2, dtype=torch.float32, device="cuda")
        return flat[2:].view(*shape)
    return one32((n, n)), one32((n, n)), one32((n, n, 2))


@pytest.mark.parametrize("pattern,r", ALL)
@pytest.mark.parametrize("mode", ["depth1", "depth4", "whole", "tuned"])
def test_odd_n_fp64_bit_exact(cuda, pattern, r, mode):
    n, k = 203, 9
    _, ref = po.run(pattern, r, n, k)
    in_a, in_b, out = kg.alloc(n, kg.FP64)
    kg.init(in_a, out)
    kw = {"depth1": {}, "depth4": {"depth": 4}, "whole": {"whole": True}, "tuned": {"tuned": True}}[mode]
    res = kg.run(pattern, r, k, in_a, in_b, out, **kw)
    assert np.array_equal(bits(out.cpu().numpy()), bits(ref))
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    assert np.array_equal(res.final_in.cpu().numpy(), (ii + jj + k + 1).astype(np.float64))


@pytest.mark.parametrize("pattern,r", [(kg.STAR, 2), (kg.GRID, 3), (kg.STAR, 5)])
@pytest.mark.parametrize("dtype", [kg.FP64, kg.FP32C])
@pytest.mark.parametrize("graph", [False, True])
def test_misaligned_buffers(cuda, pattern, r, dtype, graph):
    n, k = 128, 7
    _, ref = po.run(pattern, r, n, k)
    in_a, in_b, out = misaligned(cuda, n, dtype)
    assert in_a.data_ptr() % 16 == 8
    kg.init(in_a, out)
    res = kg.run(pattern, r, k, in_a, in_b, out, graph=graph, depth=2)
    got = out.cpu().numpy()
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    if dtype == kg.FP64:
        assert np.array_equal(bits(got), bits(ref))
    else:
        g64 = got[..., 0].astype(np.float64) + got[..., 1].astype(np.float64)
        inner = (slice(r, n - r), slice(r, n - r))
        assert (np.abs(g64[inner] - ref[inner]) / np.abs(ref[inner])).max() <= 1e-6
        assert np.all(g64[:r] == 0) and np.all(g64[n - r:] == 0)
    want = (ii + jj + k + 1).astype(np.float64)
    assert np.array_equal(res.final_in.cpu().numpy().astype(np.float64), want)
    assert abs(kg.norm(r, out) - 2.0 * (k + 1)) <= 1e-8


@pytest.mark.parametrize("n", [130, 1001])
@pytest.mark.parametrize("depth", [1, 8])
def test_ragged_fp32c_error_bound(cuda, n, depth):
    """FP32C with n not a multiple of 4 (the FP32 vector width)."""
    r, k = 2, 12
    _, ref = po.run(kg.STAR, r, n, k)
    in_a, in_b, out = kg.alloc(n, kg.FP32C)
    kg.init(in_a, out)
    res = kg.run(kg.STAR, r, k, in_a, in_b, out, depth=depth)
    got = out.cpu().numpy()
    g64 = got[..., 0].astype(np.float64) + got[..., 1].astype(np.float64)
    inner = (slice(r, n - r), slice(r, n - r))
    assert (np.abs(g64[inner] - ref[inner]) / np.abs(ref[inner])).max() <= 1e-6
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    assert np.array_equal(res.final_in.cpu().numpy(), (ii + jj + k + 1).astype(np.float32))


def test_long_run(cuda):
    """5000 applications on an odd n, one launch each and all in one launch: bit-exact."""
    n, r, k = 61, 2, 5000
    _, ref = po.run(kg.STAR, r, n, k)
    in_a, in_b, out = kg.alloc(n, kg.FP64)
    kg.init(in_a, out)
    res = kg.run(kg.STAR, r, k, in_a, in_b, out)
    assert np.array_equal(bits(out.cpu().numpy()), bits(ref))
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    assert np.array_equal(res.final_in.cpu().numpy(), (ii + jj + k + 1).astype(np.float64))
    kg.init(in_a, out)
    res = kg.run(kg.STAR, r, k, in_a, in_b, out, whole=True)
    assert np.array_equal(bits(out.cpu().numpy()), bits(ref))
    assert np.array_equal(res.final_in.cpu().numpy(), (ii + jj + k + 1).astype(np.float64))


@pytest.mark.parametrize("pattern,r", [(kg.STAR, 1), (kg.GRID, 2), (kg.STAR, 4)])
@pytest.mark.parametrize("dtype", [kg.FP64, kg.FP32C])
def test_plain_tiles_match_generic(cuda, pattern, r, dtype):
    """Same inputs through the plain-staged tiles and through the generic kernels: FP64 bit for
    bit; FP32C each within the bound of the oracle."""
    n, k = 301, 5
    outs = []
    for choice in (kg.KERNEL_AUTO, kg.KERNEL_GENERIC):
        prev = kg.set_kernel(choice)
        try:
            in_a, in_b, out = kg.alloc(n, dtype)
            kg.init(in_a, out)
            kg.run(pattern, r, k, in_a, in_b, out)
            outs.append(out.cpu().numpy())
        finally:
            kg.set_kernel(prev)
    if dtype == kg.FP64:
        assert np.array_equal(bits(outs[0]), bits(outs[1]))
    else:
        _, ref = po.run(pattern, r, n, k)
        inner = (slice(r, n - r), slice(r, n - r))
        for o in outs:
            g = o[..., 0].astype(np.float64) + o[..., 1].astype(np.float64)
            assert (np.abs(g[inner] - ref[inner]) / np.abs(ref[inner])).max() <= 1e-6


def test_tuner_on_odd_n(cuda):
    t = kg.tune(kg.STAR, 2, 203, kg.FP64, force=True)
    assert t["kernel"] in ("plain", "generic") and t["depth"] in (0, 1, 2, 4, 8)


def test_odd_n_random_fields(cuda):
    """Arbitrary in and out on an odd n: the batched kernel's certification falls back to the
    strict binary64 order where the fields are not whole numbers."""
    n, r, k = 157, 3, 4
    rng = np.random.default_rng(157)
    a = rng.standard_normal((n, n)) * 1e3
    o = rng.standard_normal((n, n))
    in_a = cuda.from_numpy(a.copy()).cuda()
    in_b = cuda.empty_like(in_a)
    out = cuda.from_numpy(o.copy()).cuda()
    res = kg.run(kg.STAR, r, k, in_a, in_b, out, depth=4)
    cur = a.copy()
    for _ in range(k + 1):
        po.apply(kg.STAR, r, cur, o)
        cur = cur + 1.0
    assert np.array_equal(bits(out.cpu().numpy()), bits(o))
    assert np.array_equal(bits(res.final_in.cpu().numpy()), bits(cur))


@pytest.mark.parametrize("pattern,r", [(kg.STAR, 1), (kg.STAR, 2), (kg.GRID, 1), (kg.STAR, 3), (kg.GRID, 5)])
@pytest.mark.parametrize("steps", [1, 2, 8])
@pytest.mark.parametrize("kind", ["small_int", "dyadic", "wide_int", "random"])
def test_apply_steps_odd_n(cuda, pattern, r, steps, kind):
    """prk_gb300_stencil_steps on an odd n, each exact route (FP32, integer, whole-number products,
    strict): the bits of `steps` single applications."""
    n = 157
    rng = np.random.default_rng(steps * 100 + r + len(kind))
    if kind == "small_int":
        a = rng.integers(-2**19, 2**19, (n, n)).astype(np.float64)
    elif kind == "dyadic":
        a = rng.integers(-2**20, 2**20, (n, n)) * 2.0 ** -9
    elif kind == "wide_int":
        a = rng.integers(-2**40, 2**40, (n, n)).astype(np.float64)
    else:
        a = rng.standard_normal((n, n)) * np.exp2(rng.integers(-10, 10, (n, n)))
    o = rng.standard_normal((n, n))
    want_in, want_out = a.copy(), o.copy()
    for _ in range(steps):
        po.apply(pattern, r, want_in, want_out)
        want_in = want_in + 1.0
    in_ = cuda.from_numpy(a).cuda()
    out = cuda.from_numpy(o.copy()).cuda()
    nxt = cuda.empty_like(in_)
    kg.apply_steps(pattern, r, steps, in_, out, nxt)
    kg.status()
    assert np.array_equal(bits(out.cpu().numpy()), bits(want_out))
    assert np.array_equal(bits(nxt.cpu().numpy()), bits(want_in))
    assert np.array_equal(in_.cpu().numpy(), a)


@pytest.mark.parametrize("pattern,r", [(kg.STAR, 2), (kg.GRID, 3)])
@pytest.mark.parametrize("mode", ["depth1", "whole"])
def test_full_size_odd_n(cuda, pattern, r, mode):
    """n=16383 (odd, the headline size less one), 100 iterations, FP64: norm check, sampled points
    against the per-point oracle (bit-exact), and the final `in` field."""
    n, K = 16383, 100
    in_a, in_b, out = kg.alloc(n, kg.FP64)
    kg.init(in_a, out)
    res = kg.run(pattern, r, K, in_a, in_b, out, whole=mode == "whole")
    assert abs(kg.norm(r, out) - 2.0 * (K + 1)) <= 1e-8
    rng = np.random.default_rng(16383 + r)
    pts = [(r, r), (n - r - 1, n - r - 1), (r, n - r - 1), (n - r - 1, r), (8191, 8192)] + \
          [tuple(int(x) for x in rng.integers(r, n - r, 2)) for _ in range(40)]
    idx = cuda.tensor([i * n + j for i, j in pts], device="cuda")
    got = out.reshape(-1)[idx].cpu().numpy()
    for (i, j), v in zip(pts, got):
        assert v == po.point(pattern, r, n, K + 1, i, j), (i, j)
    fin = res.final_in.reshape(-1)[idx].cpu().numpy()
    assert all(f == i + j + K + 1 for (i, j), f in zip(pts, fin))
    del in_a, in_b, out, res
    cuda.cuda.empty_cache()


@pytest.mark.parametrize("n", [203, 1001])
@pytest.mark.parametrize("dtype", [kg.FP64, kg.FP32C])
@pytest.mark.parametrize("pattern,r", [(kg.STAR, 2), (kg.GRID, 3)])
def test_run_host_odd_n_banded(cuda, n, dtype, pattern, r):
    """prk_gb300_run_host on an odd n: bands of plain-staged tiles (n=1001: eight bands of 128 rows,
    the last 105), each carrying every application, against the oracle and the generic kernels'
    unbanded run."""
    k = 7
    _, ref = po.run(pattern, r, n, k)
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    if dtype == kg.FP64:
        h_in = (ii + jj).astype(np.float64)
        h_out = np.zeros((n, n))
    else:
        h_in = (ii + jj).astype(np.float32)
        h_out = np.zeros((n, n, 2), np.float32)
    h_fin = np.empty_like(h_in)
    res = kg.run_host(pattern, r, k, h_in, h_out, h_fin)
    inner = (slice(r, n - r), slice(r, n - r))
    if dtype == kg.FP64:
        assert np.array_equal(bits(h_out), bits(ref))
    else:
        got = h_out.astype(np.float64).sum(axis=-1)
        assert (np.abs(got[inner] - ref[inner]) / np.abs(ref[inner])).max() <= 1e-6
    assert np.array_equal(h_fin, h_in + h_in.dtype.type(k + 1))
    assert abs(res["norm"] - 2.0 * (k + 1)) <= 1e-8
    assert res["kernel_s"] > 0
    prev = kg.set_kernel(kg.KERNEL_GENERIC)
    try:
        h_out2 = np.zeros_like(h_out)
        kg.run_host(pattern, r, k, h_in, h_out2)
    finally:
        kg.set_kernel(prev)
    if dtype == kg.FP64:
        assert np.array_equal(bits(h_out2), bits(h_out))


def test_tuned_run_with_generic_kernels_only(cuda):
    """A tuned run while the generic kernels are selected process-wide: a cached choice of the whole
    run in one launch (a tile-kernel form) falls back to one application per launch."""
    n, r, k = 203, 2, 5
    kg.tune(kg.STAR, r, n, kg.FP64)
    _, ref = po.run(kg.STAR, r, n, k)
    prev = kg.set_kernel(kg.KERNEL_GENERIC)
    try:
        in_a, in_b, out = kg.alloc(n, kg.FP64)
        kg.init(in_a, out)
        kg.run(kg.STAR, r, k, in_a, in_b, out, tuned=True)
    finally:
        kg.set_kernel(prev)
    assert np.array_equal(bits(out.cpu().numpy()), bits(ref))
