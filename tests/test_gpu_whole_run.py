"""Whole runs in one launch per tile (PRK_RUN_WHOLE, the run-time-depth tile kernel) and the banded
host-buffer run built on it: the results must be those of one application per launch, bit for bit
in FP64 and within the 1e-6 bound in FP32C, for every stencil and data kind, including runs deep
enough to leave the FP32 route and ragged last bands."""
import numpy as np
import pytest

import kernels_gb300 as kg
from oracle import prk_oracle as po

pytestmark = pytest.mark.gpu

ALL = [(p, r) for p in (kg.STAR, kg.GRID) for r in range(1, 6)]


def bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


@pytest.mark.parametrize("pattern,r", ALL)
def test_whole_run_fp64_bit_exact(cuda, pattern, r):
    n, k = 264, 11
    _, ref = po.run(pattern, r, n, k)
    in_a, in_b, out = kg.alloc(n, kg.FP64)
    kg.init(in_a, out)
    res = kg.run(pattern, r, k, in_a, in_b, out, whole=True)
    assert np.array_equal(bits(out.cpu().numpy()), bits(ref))
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    assert np.array_equal(res.final_in.cpu().numpy(), (ii + jj + k + 1).astype(np.float64))


@pytest.mark.parametrize("pattern,r", [(kg.STAR, 1), (kg.STAR, 2), (kg.GRID, 1), (kg.STAR, 3), (kg.GRID, 2)])
@pytest.mark.parametrize("kind", ["small_int", "dyadic", "wide_int", "random"])
@pytest.mark.parametrize("out_kind", ["zero", "units", "random"])
def test_whole_run_matches_single_applications(cuda, pattern, r, kind, out_kind):
    """Arbitrary in and out: each exact route (FP32, integer, strict) and the integer-held out
    (taken for zero and whole-unit out, refused for random out)."""
    n, k = 192, 6
    rng = np.random.default_rng(r * 10 + len(kind) + len(out_kind))
    if kind == "small_int":
        a = rng.integers(-2**19, 2**19, (n, n)).astype(np.float64)
    elif kind == "dyadic":
        a = rng.integers(-2**20, 2**20, (n, n)) * 2.0 ** -9
    elif kind == "wide_int":
        a = rng.integers(-2**40, 2**40, (n, n)).astype(np.float64)
    else:
        a = rng.standard_normal((n, n)) * np.exp2(rng.integers(-10, 10, (n, n)))
    if out_kind == "zero":
        o = np.zeros((n, n))
    elif out_kind == "units":
        o = rng.integers(-2**17, 2**17, (n, n)) * 0.125
    else:
        o = rng.standard_normal((n, n))
    want_in, want_out = a.copy(), o.copy()
    for _ in range(k + 1):
        po.apply(pattern, r, want_in, want_out)
        want_in = want_in + 1.0
    in_a = cuda.from_numpy(a).cuda()
    in_b = cuda.empty_like(in_a)
    out = cuda.from_numpy(o.copy()).cuda()
    res = kg.run(pattern, r, k, in_a, in_b, out, whole=True)
    kg.status()
    assert np.array_equal(bits(out.cpu().numpy()), bits(want_out))
    assert np.array_equal(bits(res.final_in.cpu().numpy()), bits(want_in))


@pytest.mark.parametrize("pattern,r", ALL)
def test_whole_run_fp32c_bound(cuda, pattern, r):
    n, k = 264, 19
    _, ref = po.run(pattern, r, n, k)
    in_a, in_b, out = kg.alloc(n, kg.FP32C)
    kg.init(in_a, out)
    kg.run(pattern, r, k, in_a, in_b, out, whole=True)
    got = out.cpu().numpy().astype(np.float64)
    got = got[..., 0] + got[..., 1]
    inner = (slice(r, n - r), slice(r, n - r))
    assert (np.abs(got[inner] - ref[inner]) / np.abs(ref[inner])).max() <= 1e-6


def test_whole_run_deeper_than_the_fp32_route(cuda):
    """66000 applications in one launch: past the FP32 route's bound the tile takes the strict
    route, and the bits equal those of launches of depth 8."""
    n, k = 64, 66000
    a = kg.alloc(n, kg.FP64)
    b = kg.alloc(n, kg.FP64)
    kg.init(a[0], a[2])
    kg.init(b[0], b[2])
    kg.run(kg.STAR, 2, k, a[0], a[1], a[2], whole=True)
    kg.run(kg.STAR, 2, k, b[0], b[1], b[2], depth=8)
    assert np.array_equal(bits(a[2].cpu().numpy()), bits(b[2].cpu().numpy()))
    assert abs(kg.norm(2, a[2]) - 2.0 * (k + 1)) <= 1e-8


@pytest.mark.parametrize("n", [600, 1000, 2048])
@pytest.mark.parametrize("pattern,r", [(kg.STAR, 2), (kg.GRID, 3), (kg.STAR, 5)])
def test_run_host_banded_fp64(cuda, n, pattern, r):
    """Several bands, a ragged last band (600, 1000), pageable and pinned host buffers."""
    k = 7
    _, ref = po.run(pattern, r, n, k)
    for pinned in (False, True):
        h_in = cuda.from_numpy(np.add.outer(np.arange(n), np.arange(n)).astype(np.float64))
        h_out = cuda.zeros((n, n), dtype=cuda.float64)
        h_fin = cuda.empty((n, n), dtype=cuda.float64)
        if pinned:
            h_in, h_out, h_fin = h_in.pin_memory(), h_out.pin_memory(), h_fin.pin_memory()
        res = kg.run_host(pattern, r, k, h_in, h_out, h_fin)
        assert np.array_equal(bits(h_out.numpy()), bits(ref))
        assert np.array_equal(h_fin.numpy(), h_in.numpy() + k + 1)
        assert abs(res["norm"] - 2.0 * (k + 1)) <= 1e-8
        assert res["kernel_s"] > 0


@pytest.mark.parametrize("pattern,r", [(kg.STAR, 2), (kg.GRID, 4)])
def test_run_host_banded_fp32c(cuda, pattern, r):
    n, k = 1000, 9
    _, ref = po.run(pattern, r, n, k)
    h_in = np.add.outer(np.arange(n), np.arange(n)).astype(np.float32)
    h_out = np.zeros((n, n, 2), np.float32)
    h_fin = np.empty_like(h_in)
    res = kg.run_host(pattern, r, k, h_in, h_out, h_fin)
    got = h_out.astype(np.float64)
    got = got[..., 0] + got[..., 1]
    inner = (slice(r, n - r), slice(r, n - r))
    assert (np.abs(got[inner] - ref[inner]) / np.abs(ref[inner])).max() <= 1e-6
    assert np.array_equal(h_fin, h_in + np.float32(k + 1))
    assert abs(res["norm"] - 2.0 * (k + 1)) <= 1e-8


def test_whole_run_rejections(cuda):
    in_a, in_b, out = kg.alloc(63, kg.FP64)  # odd n: the generic kernels have no whole-run form
    prev = kg.set_kernel(kg.KERNEL_GENERIC)
    try:
        with pytest.raises(kg.PrkError):
            kg.run(kg.STAR, 2, 3, in_a, in_b, out, whole=True)
    finally:
        kg.set_kernel(prev)
    in_a, in_b, out = kg.alloc(64, kg.FP64)
    with pytest.raises(kg.PrkError):
        kg.run(kg.STAR, 2, 3, in_a, None, out, whole=True, unfused=True)


@pytest.mark.parametrize("n", [8, 64, 130])
@pytest.mark.parametrize("dtype", [kg.FP64, kg.FP32C])
def test_run_host_smallest_shapes(cuda, n, dtype):
    """One band (n below the band height), the smallest TMA shapes, and a ragged FP32C size."""
    if dtype == kg.FP32C and n % 4:
        n += 4 - n % 4
    r, k = 1, 3
    _, ref = po.run(kg.STAR, r, n, k)
    if dtype == kg.FP64:
        h_in = np.add.outer(np.arange(n), np.arange(n)).astype(np.float64)
        h_out = np.zeros((n, n))
    else:
        h_in = np.add.outer(np.arange(n), np.arange(n)).astype(np.float32)
        h_out = np.zeros((n, n, 2), np.float32)
    res = kg.run_host(kg.STAR, r, k, h_in, h_out)
    got = h_out if dtype == kg.FP64 else h_out.astype(np.float64).sum(axis=-1)
    inner = (slice(r, n - r), slice(r, n - r))
    if dtype == kg.FP64:
        assert np.array_equal(bits(got), bits(ref))
    else:
        assert (np.abs(got[inner] - ref[inner]) / np.abs(ref[inner])).max() <= 1e-6
    assert abs(res["norm"] - 2.0 * (k + 1)) <= 1e-8


def test_whole_run_of_one_timed_application(cuda):
    n, k = 96, 1
    _, ref = po.run(kg.GRID, 2, n, k)
    in_a, in_b, out = kg.alloc(n, kg.FP64)
    kg.init(in_a, out)
    kg.run(kg.GRID, 2, k, in_a, in_b, out, whole=True)
    assert np.array_equal(bits(out.cpu().numpy()), bits(ref))


@pytest.mark.parametrize("pattern,r", [(kg.STAR, 2), (kg.GRID, 3)])
def test_whole_run_full_size_sampled(cuda, pattern, r):
    """n=16384, 100 timed iterations in one launch per tile (the FP32 route for star R=2, integer
    products for grid R=3): the norm, sampled points against the per-point oracle bit for bit,
    tile corners included, and the final `in`."""
    n, K = 16384, 100
    in_a, in_b, out = kg.alloc(n, kg.FP64)
    kg.init(in_a, out)
    res = kg.run(pattern, r, K, in_a, in_b, out, whole=True)
    assert abs(kg.norm(r, out) - 2.0 * (K + 1)) <= 1e-8
    rng = np.random.default_rng(17 + r)
    pts = [(r, r), (n - r - 1, n - r - 1), (r, n - r - 1), (31, 63), (32, 64), (8191, 8192)] + \
          [tuple(int(x) for x in rng.integers(r, n - r, 2)) for _ in range(60)]
    idx = cuda.tensor([i * n + j for i, j in pts], device="cuda")
    got = out.reshape(-1)[idx].cpu().numpy()
    for (i, j), v in zip(pts, got):
        assert v == po.point(pattern, r, n, K + 1, i, j), (i, j)
    fin = res.final_in.reshape(-1)[idx].cpu().numpy()
    assert all(f == i + j + K + 1 for (i, j), f in zip(pts, fin))


def test_run_host_banded_full_size_sampled(cuda):
    """The banded host-buffer run at n=16384 with pinned buffers, sampled against the oracle."""
    n, K, r = 16384, 20, 2
    idx = cuda.arange(n, dtype=cuda.float64)
    h_in = (idx[:, None] + idx[None, :]).pin_memory()
    h_out = cuda.zeros((n, n), dtype=cuda.float64).pin_memory()
    res = kg.run_host(kg.STAR, r, K, h_in, h_out)
    assert abs(res["norm"] - 2.0 * (K + 1)) <= 1e-8
    rng = np.random.default_rng(5)
    pts = [(r, r), (n - r - 1, n - r - 1), (511, 1000), (512, 1000), (513, 7)] + \
          [tuple(int(x) for x in rng.integers(r, n - r, 2)) for _ in range(40)]
    out = h_out.numpy()
    for i, j in pts:
        assert out[i, j] == po.point(kg.STAR, r, n, K + 1, i, j), (i, j)
