"""Batched grids (one persistent kernel over the tiles of many grids, device work queue, CUDA
graph) and the autotuner: every grid of a mixed batch must match its own oracle run exactly
(FP64) or within the 1e-6 bound (FP32C), whatever depth, graph or tuning is used."""
import numpy as np
import pytest

import kernels_gb300 as kg
from kernels_gb300.workloads import batch_specs
from oracle import prk_oracle as po

pytestmark = pytest.mark.gpu

MIXED = [(kg.STAR, 1, 37), (kg.GRID, 5, 11), (kg.STAR, 2, 130), (kg.GRID, 2, 257), (kg.STAR, 5, 64),
         (kg.GRID, 1, 1000), (kg.STAR, 3, 513), (kg.GRID, 4, 96), (kg.STAR, 4, 300), (kg.GRID, 3, 45),
         (kg.STAR, 2, 1), (kg.GRID, 1, 3)]


def make_batch(torch, specs, dtype, **kw):
    grids = []
    for p, r, n in specs:
        in_a, in_b, out = kg.alloc(n, dtype)
        kg.init(in_a, out)
        grids.append((p, r, in_a, in_b, out))
    return kg.Batch(grids, **kw), grids


def check_fp64(b, grids, specs, k):
    for idx, ((p, r, n), g) in enumerate(zip(specs, grids)):
        _, ref = po.run(p, r, n, k)
        got = g[4].cpu().numpy()
        assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), (p, r, n)
        ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
        assert np.array_equal(b.final_in(idx).cpu().numpy(), (ii + jj + k + 1).astype(np.float64))


VALID = [s for s in MIXED if 2 * s[1] + 1 <= s[2]]


@pytest.mark.parametrize("depth", [1, 2, 4, 8])
@pytest.mark.parametrize("graph", [False, True])
def test_mixed_batch_fp64_bit_exact(cuda, depth, graph):
    k = 9
    b, grids = make_batch(cuda, VALID, kg.FP64, depth=depth)
    b.run(k, graph=graph)
    check_fp64(b, grids, VALID, k)
    norms = b.norms()
    assert all(abs(x - 2.0 * (k + 1)) <= 1e-8 for x in norms)
    if graph:  # a second replay of the cached graph after re-initialising
        for p, r, in_a, in_b, out in grids:
            kg.init(in_a, out)
        b.run(k, graph=True)
        check_fp64(b, grids, VALID, k)
    b.close()


@pytest.mark.parametrize("graph", [False, True])
def test_mixed_batch_whole_run_fp64_bit_exact(cuda, graph):
    """Every grid's timed applications in one launch of the batched kernel per kernel family (the
    power-of-two stencils share one; every stencil with other weights has its own)."""
    k = 9
    b, grids = make_batch(cuda, VALID, kg.FP64, whole=True)
    families = {"pow2" if (p, r) in ((kg.STAR, 1), (kg.STAR, 2), (kg.GRID, 1)) else (p, r) for p, r, _ in VALID}
    assert b.launches(k) == len(families)
    b.run(k, graph=graph)
    check_fp64(b, grids, VALID, k)
    assert all(abs(x - 2.0 * (k + 1)) <= 1e-8 for x in b.norms())
    b.close()


def test_mixed_batch_whole_run_fp32c_bound(cuda):
    k = 12
    b, grids = make_batch(cuda, VALID, kg.FP32C, whole=True)
    b.run(k, graph=True)
    for (p, r, n), g in zip(VALID, grids):
        _, ref = po.run(p, r, n, k)
        got = g[4].cpu().numpy().astype(np.float64)
        got = got[..., 0] + got[..., 1]
        inner = (slice(r, n - r), slice(r, n - r))
        assert (np.abs(got[inner] - ref[inner]) / np.abs(ref[inner])).max() <= 1e-6, (p, r, n)
    b.close()


def test_mixed_batch_fp32c_bound(cuda):
    k = 12
    b, grids = make_batch(cuda, VALID, kg.FP32C, depth=4)
    b.run(k, graph=True)
    for (p, r, n), g in zip(VALID, grids):
        _, ref = po.run(p, r, n, k)
        o = g[4].cpu().numpy().astype(np.float64)
        got = o[..., 0] + o[..., 1]
        inner = (slice(r, n - r), slice(r, n - r))
        assert (np.abs(got[inner] - ref[inner]) / np.abs(ref[inner])).max() <= 1e-6
    assert all(abs(x - 2.0 * (k + 1)) <= 1e-8 for x in b.norms())
    b.close()


def test_seeded_batch_norms(cuda):
    """The first 48 grids of the seeded 256-grid configuration, tuned depths, graph: every norm
    checks against 2(K+1), and sampled points against the per-point oracle."""
    specs = batch_specs()[:48]
    k = 10
    b, grids = make_batch(cuda, specs, kg.FP64, tuned=True)
    b.run(k, graph=True)
    norms = b.norms()
    assert all(abs(x - 2.0 * (k + 1)) <= 1e-8 for x in norms)
    rng = np.random.default_rng(5)
    for (p, r, n), g in zip(specs, grids):
        for _ in range(3):
            i, j = (int(x) for x in rng.integers(r, n - r, 2))
            assert float(g[4][i, j]) == po.point(p, r, n, k + 1, i, j)
    b.close()


def test_batch_rejects_bad_grids(cuda):
    in_a, in_b, out = kg.alloc(16)
    with pytest.raises(kg.PrkError):
        kg.Batch([(kg.STAR, 9, in_a, in_b, out)])
    with pytest.raises(kg.PrkError):
        kg.Batch([])


def test_tuner_choice_is_cached_and_used(cuda, tmp_path, monkeypatch):
    t1 = kg.tune(kg.STAR, 2, 1024, kg.FP64, force=True)
    assert t1["depth"] in (0, 1, 2, 4, 8) and t1["kernel"] in ("tma", "generic")  # 0: whole run in one launch
    assert t1["seconds_per_application"] > 0 and not t1["from_cache"]
    t2 = kg.tune(kg.STAR, 2, 1024, kg.FP64)
    assert t2["from_cache"] and t2["depth"] == t1["depth"]
    tb = kg.tune(kg.GRID, 3, 515, kg.FP32C, batch=True)
    assert tb["kernel"] == "batched"
    # a tuned run gives the reference's bits
    n, k = 1024, 9
    _, ref = po.run(kg.STAR, 2, n, k)
    in_a, in_b, out = kg.alloc(n)
    kg.init(in_a, out)
    kg.run(kg.STAR, 2, k, in_a, in_b, out, tuned=True)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), ref.view(np.uint64))
