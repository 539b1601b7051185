"""The table route of the strict FP64 stencils (star R=3..5, grid R=2..5) against the oracle, bit for
bit, on whole-number fields built to reach its edges: products from a per-tile table of fl(|w| * v),
the first part of each chain in 96-bit fixed point, the rest on the binary64 pipe.

Fields: small ranges of both signs with zeros (every tile takes the route), ranges just inside and
just outside the table's 128 values (some tiles take it, the others the product route), all zeros
with -0 in out (the sign of a zero sum), large magnitudes near 2^19, and random whole numbers.
Multi-application launches (depths 2, 4, 8 and whole runs) advance the tile and rebuild the table
when the values outgrow it."""
import numpy as np
import pytest

import kernels_gb300 as kg
from oracle import prk_oracle as po

pytestmark = pytest.mark.gpu

STRICT = [(kg.STAR, 3), (kg.STAR, 4), (kg.STAR, 5), (kg.GRID, 2), (kg.GRID, 3), (kg.GRID, 4), (kg.GRID, 5)]


def whole_fields(n, rng):
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    f = {}
    small = rng.integers(-40, 40, (n, n)).astype(np.float64)
    small[rng.random((n, n)) < 0.2] = 0.0
    f["small_signed_zeros"] = small
    f["range_127"] = (rng.integers(0, 128, (n, n)) + 5000).astype(np.float64)
    f["range_129"] = (rng.integers(0, 130, (n, n)) - 70000).astype(np.float64)
    f["near_2_19"] = (rng.integers(-60, 60, (n, n)) + (2 ** 19 - 100) * np.sign(ii - jj + 0.5)).astype(np.float64)
    f["random_whole"] = rng.integers(-2 ** 18, 2 ** 18, (n, n)).astype(np.float64)
    f["diagonal"] = (ii - jj).astype(np.float64)  # the PRK field's mirror: negative, zero and positive
    return f


def same_bits(x, y):
    return np.array_equal(x.view(np.uint64), y.view(np.uint64))


@pytest.mark.parametrize("pattern,r", STRICT)
def test_one_application_bit_exact(cuda, pattern, r):
    n = 300
    rng = np.random.default_rng(31 * r + pattern)
    o = rng.standard_normal((n, n)) * 100.0
    o[r + 2, r + 3] = -0.0
    o[r + 9, r + 9] = 0.0
    for name, a in whole_fields(n, rng).items():
        want = o.copy()
        po.apply(pattern, r, a, want)
        in_ = cuda.from_numpy(a).cuda()
        out = cuda.from_numpy(o.copy()).cuda()
        nxt = cuda.empty_like(in_)
        kg.apply(pattern, r, in_, out, in_next=nxt)
        kg.status()
        assert same_bits(out.cpu().numpy(), want), name
        assert same_bits(nxt.cpu().numpy(), a + 1.0), name


@pytest.mark.parametrize("pattern,r", STRICT)
def test_zero_fields_keep_the_sign_of_zero(cuda, pattern, r):
    """All-zero in: every product is +-0, the chain sums to -0 exactly when all its terms are -0,
    and out = -0 stays -0 only then."""
    n = 128
    a = np.zeros((n, n))
    o = np.zeros((n, n))
    o[::2] = -0.0
    want = o.copy()
    po.apply(pattern, r, a, want)
    in_ = cuda.from_numpy(a).cuda()
    out = cuda.from_numpy(o.copy()).cuda()
    kg.apply(pattern, r, in_, out, in_next=cuda.empty_like(in_))
    assert same_bits(out.cpu().numpy(), want)


@pytest.mark.parametrize("pattern,r", STRICT)
@pytest.mark.parametrize("depth", [2, 4, 8, "whole"])
def test_multi_application_bit_exact(cuda, pattern, r, depth):
    """Applications on a tile held in shared memory; 40 of them in one launch for the whole run,
    which rebuilds the table as the values climb past its 128 entries."""
    n, apps = 260, 40 if depth == "whole" else depth
    rng = np.random.default_rng(7 * r + pattern + (0 if depth == "whole" else depth))
    a = rng.integers(-50, 50, (n, n)).astype(np.float64)
    o = rng.standard_normal((n, n))
    want_in, want_out = a.copy(), o.copy()
    for _ in range(apps):
        po.apply(pattern, r, want_in, want_out)
        want_in += 1.0
    in_a = cuda.from_numpy(a).cuda()
    in_b = cuda.empty_like(in_a)
    out = cuda.from_numpy(o.copy()).cuda()
    if depth == "whole":
        kg.run(pattern, r, apps - 1, in_a, in_b, out, whole=True)  # application 0, then the rest in one launch
        fin = None
    else:
        kg.apply_steps(pattern, r, depth, in_a, out, in_b)
        fin = in_b
    kg.status()
    assert same_bits(out.cpu().numpy(), want_out)
    if fin is not None:
        assert same_bits(fin.cpu().numpy(), want_in)


@pytest.mark.parametrize("pattern,r", STRICT)
def test_prk_run_against_reference_fixture_sizes(cuda, pattern, r):
    """A PRK run (in = i+j) at n=1030 and n=4096, 12 iterations: the table route on every tile."""
    for n in (1030, 4096):
        _, ref = po.run(pattern, r, n, 12)
        in_a, in_b, out = kg.alloc(n, kg.FP64)
        kg.init(in_a, out)
        kg.run(pattern, r, 12, in_a, in_b, out)
        assert same_bits(out.cpu().numpy(), ref), n
