"""The FP64 TMA kernels against the oracle, bit for bit, on data built to exercise the certified
integer route of the power-of-two stencils (star R=1,2, grid R=1) and its per-tile fallback to the
strict binary64 route: integer and dyadic fields, wide and narrow integer ranges, negative values,
values at the certification bounds, and tiles holding -0.0, NaN, infinities or subnormals."""
import numpy as np
import pytest

import kernels_gb300 as kg
from oracle import prk_oracle as po

pytestmark = pytest.mark.gpu

POW2 = [(kg.STAR, 1), (kg.STAR, 2), (kg.GRID, 1)]


def one_step(torch, pattern, r, a, o, kernel=kg.KERNEL_AUTO):
    prev = kg.set_kernel(kernel)
    try:
        in_ = torch.from_numpy(a).cuda()
        out = torch.from_numpy(o.copy()).cuda()
        nxt = torch.empty_like(in_)
        kg.apply(pattern, r, in_, out, in_next=nxt)
        kg.status()
        return out.cpu().numpy(), nxt.cpu().numpy()
    finally:
        kg.set_kernel(prev)


def same_bits(x, y):
    """Bitwise equality, except that NaNs only need to sit at the same places."""
    nx, ny = np.isnan(x), np.isnan(y)
    return np.array_equal(nx, ny) and np.array_equal(x[~nx].view(np.uint64), y[~ny].view(np.uint64))


def fields(n, rng):
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    f = {}
    f["prk"] = (ii + jj).astype(np.float64)
    f["wide_int"] = (ii * 3.0 + jj) * 2.0 ** 33 + rng.integers(-2**20, 2**20, (n, n))
    f["dyadic"] = rng.integers(-2**22, 2**22, (n, n)) * 2.0 ** -17
    f["negative"] = -(ii + 2.0 * jj) - 0.5
    f["random"] = rng.standard_normal((n, n)) * np.exp2(rng.integers(-30, 30, (n, n)))
    big = rng.integers(-2**47, 2**47, (n, n)).astype(np.float64)  # near the 2^53 / coefficient bound
    f["near_bound"] = big
    mixed = (ii + jj).astype(np.float64)
    mixed[5, 7] = -0.0
    mixed[40, 100] = np.nan
    mixed[70, 3] = np.inf
    mixed[100, 200] = -np.inf
    mixed[130, 66] = 5e-324  # subnormal
    mixed[150, 150] = 2.0 ** 70
    f["mixed_specials"] = mixed
    return f


@pytest.mark.parametrize("pattern,r", POW2 + [(kg.STAR, 3), (kg.GRID, 2)])
def test_fused_step_bit_exact_on_all_field_kinds(cuda, pattern, r):
    n = 256
    rng = np.random.default_rng(17 * r + pattern)
    o = rng.standard_normal((n, n)) * 10.0
    o[3, 3] = -0.0
    for name, a in fields(n, rng).items():
        want_out = o.copy()
        po.apply(pattern, r, a, want_out)
        got_out, got_next = one_step(cuda, pattern, r, a, o)
        assert same_bits(got_out, want_out), name
        assert same_bits(got_next, a + 1.0), name


@pytest.mark.parametrize("pattern,r", POW2)
@pytest.mark.parametrize("n", [1000, 1030, 4096])
def test_tma_and_generic_agree_and_match_reference_runs(cuda, pattern, r, n):
    """Whole PRK runs (in=i+j, out=0) through both kernel families against the strict oracle."""
    _, ref = po.run(pattern, r, n, 7)
    for kern in (kg.KERNEL_TMA, kg.KERNEL_GENERIC):
        prev = kg.set_kernel(kern)
        try:
            in_a, in_b, out = kg.alloc(n, kg.FP64)
            kg.init(in_a, out)
            kg.run(pattern, r, 7, in_a, in_b, out)
            assert np.array_equal(out.cpu().numpy().view(np.uint64), ref.view(np.uint64)), kern
        finally:
            kg.set_kernel(prev)


def test_tma_required_rejects_ineligible_shapes(cuda):
    prev = kg.set_kernel(kg.KERNEL_TMA)
    try:
        a = cuda.zeros((63, 63), dtype=cuda.float64, device="cuda")  # odd n: rows not 16-byte multiples
        o = cuda.zeros_like(a)
        with pytest.raises(kg.PrkError):
            kg.apply(kg.STAR, 2, a, o, in_next=cuda.zeros_like(a))
    finally:
        kg.set_kernel(prev)


@pytest.mark.parametrize("pattern", [kg.STAR, kg.GRID])
@pytest.mark.parametrize("r", range(1, 6))
def test_fp32c_tma_within_bound(cuda, pattern, r):
    n, k = 512, 20
    _, ref = po.run(pattern, r, n, k)
    prev = kg.set_kernel(kg.KERNEL_TMA)
    try:
        in_a, in_b, out = kg.alloc(n, kg.FP32C)
        kg.init(in_a, out)
        res = kg.run(pattern, r, k, in_a, in_b, out)
    finally:
        kg.set_kernel(prev)
    got = out.cpu().numpy().astype(np.float64)
    got = got[..., 0] + got[..., 1]
    inner = (slice(r, n - r), slice(r, n - r))
    rel = np.abs(got[inner] - ref[inner]) / np.abs(ref[inner])
    assert rel.max() <= 1e-6
    assert np.all(got[:r] == 0) and np.all(got[:, n - r:] == 0)
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    assert np.array_equal(res.final_in.cpu().numpy(), (ii + jj + k + 1).astype(np.float32))
