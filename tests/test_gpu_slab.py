"""The row-slab entry points (prk_gb300_slab_run, prk_gb300_slab_norm) on the GPU.

A grid split across P ranks is emulated in one process on one GPU: every slab has its own buffers,
and before each launch the halo rows are copied from the neighbouring slabs' owned rows with plain
device copies ordered by the host (no kernel waits on another). The owned rows gathered from the
slabs must equal the single-grid results: the oracle bit for bit in FP64 on the reference's CI cases
and odd sizes (plain-staged tiles), the whole-grid GPU run bit for bit at n=4096, and FP32C within
1e-6 of the FP64 oracle. The slabs' norm sums, added up, give the grid's norm. SlabRun on a single
rank runs the same entry points through kernels_gb300.decomp.
"""
import numpy as np
import pytest

import kernels_gb300 as kg
from kernels_gb300.decomp import DeviceBackend, Slab, SlabRun
from oracle import prk_oracle as po

pytestmark = pytest.mark.gpu

FP32C_REL_TOL = 1e-6


def copy_rows(dst_slab, dst, src_slab, src, g0, g1):
    """Grid rows [g0, g1) from one slab's buffer into another's."""
    if g1 > g0:
        dst[g0 - dst_slab.halo_begin:g1 - dst_slab.halo_begin] = src[g0 - src_slab.halo_begin:g1 - src_slab.halo_begin]


def emulated_run(torch, pattern, r, n, k, world, depth, dtype):
    """iterations = k after application 0, in launches of `depth`; returns (out, in) as float64 grids."""
    slabs = [Slab.of(n, r, q, world) for q in range(world)]
    be = DeviceBackend()
    bufs = [list(be.alloc(s, dtype)) for s in slabs]
    for s, b in zip(slabs, bufs):
        rows = torch.arange(s.row_begin, s.row_end, device="cuda", dtype=torch.float64)[:, None]
        cols = torch.arange(n, device="cuda", dtype=torch.float64)[None, :]
        b[0].zero_()
        b[0][s.own] = (rows + cols).to(b[0].dtype)
        b[2].zero_()
    cur = 0

    def launch(apps):
        nonlocal cur
        torch.cuda.synchronize()
        for q, s in enumerate(slabs):
            if q > 0:
                copy_rows(s, bufs[q][cur], slabs[q - 1], bufs[q - 1][cur], s.halo_begin, s.row_begin)
            if q < world - 1:
                copy_rows(s, bufs[q][cur], slabs[q + 1], bufs[q + 1][cur], s.row_end, s.halo_end)
        for s, b in zip(slabs, bufs):
            kg.slab_run(pattern, r, n, apps, s.row_begin, s.row_end, b[cur], b[cur ^ 1], b[2])
        cur ^= 1

    launch(1)
    left = k
    while left:
        a = min(depth, left)
        launch(a)
        left -= a
    torch.cuda.synchronize()
    out = np.zeros((n, n))
    fin = np.zeros((n, n))
    total = 0.0
    for s, b in zip(slabs, bufs):
        o = b[2][s.own].cpu().numpy()
        out[s.row_begin:s.row_end] = o if dtype == kg.FP64 else o[..., 0].astype(np.float64) + o[..., 1]
        fin[s.row_begin:s.row_end] = b[cur][s.own].cpu().numpy()
        total += kg.slab_norm(r, n, s.row_begin, s.row_end, b[2])
    return out, fin, total / float((n - 2 * r) ** 2)


@pytest.mark.parametrize("world,depth", [(1, 1), (2, 1), (3, 4), (4, 3)])
@pytest.mark.parametrize("pattern", [kg.STAR, kg.GRID])
@pytest.mark.parametrize("r", range(1, 6))
def test_slabs_fp64_match_the_oracle(cuda, world, depth, pattern, r):
    n, k = 200, 10
    out, fin, nrm = emulated_run(cuda, pattern, r, n, k, world, depth, kg.FP64)
    in_ref, out_ref = po.run(pattern, r, n, k)
    assert np.array_equal(out.view(np.uint64), out_ref.view(np.uint64))
    assert np.array_equal(fin, in_ref)
    assert abs(nrm - po.norm(r, out_ref)) <= 1e-13 * nrm
    assert abs(nrm - 2.0 * (k + 1)) <= 1e-8


@pytest.mark.parametrize("n", [37, 199, 1001])
@pytest.mark.parametrize("depth", [1, 5])
def test_slabs_odd_n_plain_staged_tiles(cuda, n, depth):
    for pattern, r in ((kg.STAR, 2), (kg.GRID, 3)):
        world = 3 if n > 40 else 2
        out, fin, nrm = emulated_run(cuda, pattern, r, n, 7, world, depth, kg.FP64)
        in_ref, out_ref = po.run(pattern, r, n, 7)
        assert np.array_equal(out.view(np.uint64), out_ref.view(np.uint64)), (n, pattern, r)
        assert np.array_equal(fin, in_ref)


@pytest.mark.parametrize("pattern,r", [(kg.STAR, 2), (kg.GRID, 1), (kg.STAR, 4), (kg.GRID, 3)])
def test_slabs_fp32c_within_bound(cuda, pattern, r):
    n, k = 1000, 10
    out, _, nrm = emulated_run(cuda, pattern, r, n, k, 3, 4, kg.FP32C)
    _, out_ref = po.run(pattern, r, n, k)
    inner = (slice(r, n - r), slice(r, n - r))
    assert np.max(np.abs(out[inner] - out_ref[inner]) / np.abs(out_ref[inner])) <= FP32C_REL_TOL
    assert abs(nrm - 2.0 * (k + 1)) <= 1e-8


def test_slabs_match_the_whole_grid_run_n4096(cuda):
    n, k, r = 4096, 20, 3
    for pattern in (kg.STAR, kg.GRID):
        out, _, _ = emulated_run(cuda, pattern, r, n, k, 5, 8, kg.FP64)
        in_a, in_b, o = kg.alloc(n)
        kg.init(in_a, o)
        kg.run(pattern, r, k, in_a, in_b, o)
        assert np.array_equal(out.view(np.uint64), o.cpu().numpy().view(np.uint64))


@pytest.mark.parametrize("dtype", [kg.FP64, kg.FP32C])
def test_slabrun_single_rank_on_device(cuda, dtype):
    """kernels_gb300.decomp.SlabRun with one rank: the whole grid as one slab, through the device
    backend; the same bits as prk_gb300_run."""
    n, k, r = 1000, 10, 2
    run = SlabRun(kg.GRID, r, n, dtype, backend=DeviceBackend(), depth=4)
    run.init()
    run.run(k)
    assert abs(run.norm() - 2.0 * (k + 1)) <= 1e-8
    in_a, in_b, o = kg.alloc(n, dtype)
    kg.init(in_a, o)
    kg.run(kg.GRID, r, k, in_a, in_b, o)
    assert cuda.equal(run.out, o)


def test_slab_rejects_bad_calls(cuda):
    in_a, in_b, o = kg.alloc(64)
    lib = kg._lib.load()
    for rb, re_ in ((-1, 10), (10, 10), (0, 65)):
        assert lib.prk_gb300_slab_run(kg.STAR, 2, 64, kg.FP64, 1, rb, re_, in_a.data_ptr(), in_b.data_ptr(),
                                      o.data_ptr(), None) == -1
    assert lib.prk_gb300_slab_run(kg.STAR, 2, 64, kg.FP64, 0, 0, 64, in_a.data_ptr(), in_b.data_ptr(),
                                  o.data_ptr(), None) == -1
    assert lib.prk_gb300_slab_run(kg.STAR, 2, 64, kg.FP64, 1, 0, 64, in_a.data_ptr(), in_a.data_ptr(),
                                  o.data_ptr(), None) == -1  # in_next overlaps in
