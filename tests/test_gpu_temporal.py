"""Temporal blocking: `steps` applications per launch on a tile held in shared memory must give
exactly what `steps` single applications give (bit for bit in FP64, within the 1e-6 bound in
FP32C), for every stencil, data kind and depth."""
import numpy as np
import pytest

import kernels_gb300 as kg
from oracle import prk_oracle as po

pytestmark = pytest.mark.gpu

ALL = [(p, r) for p in (kg.STAR, kg.GRID) for r in range(1, 6)]


@pytest.mark.parametrize("pattern,r", ALL)
@pytest.mark.parametrize("depth", [2, 4, 8])
def test_run_with_depth_fp64_bit_exact(cuda, pattern, r, depth):
    n, k = 264, 11  # 11 timed iterations: launches of `depth` plus a remainder
    _, ref = po.run(pattern, r, n, k)
    in_a, in_b, out = kg.alloc(n, kg.FP64)
    kg.init(in_a, out)
    res = kg.run(pattern, r, k, in_a, in_b, out, depth=depth)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), ref.view(np.uint64))
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    assert np.array_equal(res.final_in.cpu().numpy(), (ii + jj + k + 1).astype(np.float64))


@pytest.mark.parametrize("pattern,r", [(kg.STAR, 1), (kg.STAR, 2), (kg.GRID, 1), (kg.STAR, 3), (kg.GRID, 2)])
@pytest.mark.parametrize("steps", [2, 4, 8])
@pytest.mark.parametrize("kind", ["random", "dyadic", "wide_int"])
def test_apply_steps_matches_repeated_single_steps(cuda, pattern, r, steps, kind):
    n = 192
    rng = np.random.default_rng(steps * 100 + r)
    if kind == "random":
        a = rng.standard_normal((n, n)) * np.exp2(rng.integers(-10, 10, (n, n)))
    elif kind == "dyadic":
        a = rng.integers(-2**20, 2**20, (n, n)) * 2.0 ** -9
    else:
        a = rng.integers(-2**40, 2**40, (n, n)).astype(np.float64)
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
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want_out.view(np.uint64))
    assert np.array_equal(nxt.cpu().numpy().view(np.uint64), want_in.view(np.uint64))
    assert np.array_equal(in_.cpu().numpy(), a)  # in is left untouched


@pytest.mark.parametrize("pattern,r", ALL)
def test_run_with_depth_fp32c_bound(cuda, pattern, r):
    n, k = 264, 19
    _, ref = po.run(pattern, r, n, k)
    in_a, in_b, out = kg.alloc(n, kg.FP32C)
    kg.init(in_a, out)
    kg.run(pattern, r, k, in_a, in_b, out, depth=8)
    got = out.cpu().numpy().astype(np.float64)
    got = got[..., 0] + got[..., 1]
    inner = (slice(r, n - r), slice(r, n - r))
    assert (np.abs(got[inner] - ref[inner]) / np.abs(ref[inner])).max() <= 1e-6


def test_graph_with_depth(cuda):
    n, k = 1000, 10
    _, ref = po.run(kg.STAR, 2, n, k)
    in_a, in_b, out = kg.alloc(n, kg.FP64)
    kg.init(in_a, out)
    kg.run(kg.STAR, 2, k, in_a, in_b, out, depth=4, graph=True)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), ref.view(np.uint64))


def test_bad_depth_rejected(cuda):
    in_a, in_b, out = kg.alloc(64, kg.FP64)
    with pytest.raises(kg.PrkError):
        kg.apply_steps(kg.STAR, 2, 3, in_a, out, in_b)
    with pytest.raises(kg.PrkError):
        kg.run(kg.STAR, 2, 4, in_a, in_b, out, depth=16)


@pytest.mark.parametrize("pattern,r", ALL)
@pytest.mark.parametrize("depth", [1, 8])
def test_tall_tiles_fp64_bit_exact(cuda, pattern, r, depth):
    """The 64-row tile variant (8 rows per thread) gives the same bits as the reference."""
    n, k = 330, 9
    _, ref = po.run(pattern, r, n, k)
    in_a, in_b, out = kg.alloc(n, kg.FP64)
    kg.init(in_a, out)
    kg.run(pattern, r, k, in_a, in_b, out, depth=depth, tall=True)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("pattern", [kg.STAR, kg.GRID])
@pytest.mark.parametrize("r", [1, 3, 5])
def test_tall_tiles_fp32c_bound(cuda, pattern, r):
    n, k = 516, 9
    _, ref = po.run(pattern, r, n, k)
    in_a, in_b, out = kg.alloc(n, kg.FP32C)
    kg.init(in_a, out)
    kg.run(pattern, r, k, in_a, in_b, out, depth=4, tall=True)
    got = out.cpu().numpy().astype(np.float64)
    got = got[..., 0] + got[..., 1]
    inner = (slice(r, n - r), slice(r, n - r))
    assert (np.abs(got[inner] - ref[inner]) / np.abs(ref[inner])).max() <= 1e-6
