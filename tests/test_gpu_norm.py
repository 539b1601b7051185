"""The device L1 norm (prk_gb300_norm, Cxx11/stencil-openmp.cc:230-239) on fields beyond PRK's own.

The FP64 norm splits each |out| into a float pair from its encoding and sums pairs in two-float
arithmetic; values whose exponent lies outside that split's range go into a binary64 sum instead.
Each test compares with the exact sum (math.fsum) of the interior's absolute values over
(n-2R)^2, within 1e-13 relative, the tolerance the golden norms are held to.
"""
import math

import numpy as np
import pytest

import kernels_gb300 as kg

pytestmark = pytest.mark.gpu

REL_TOL = 1e-13


def exact_norm(a: np.ndarray, r: int) -> float:
    n = a.shape[0]
    inner = np.abs(a[r:n - r, r:n - r]).ravel()
    return math.fsum(inner.tolist()) / float((n - 2 * r) ** 2)


def device_norm(torch, a: np.ndarray, r: int) -> float:
    return kg.norm(r, torch.from_numpy(np.ascontiguousarray(a)).cuda())


@pytest.mark.parametrize("n,r", [(5, 2), (257, 1), (1024, 3), (3001, 5)])
def test_mixed_magnitudes(cuda, n, r):
    """Signs, zeros of both signs and magnitudes from 2^-300 to 2^300: every branch of the split."""
    rng = np.random.default_rng(n + r)
    a = rng.standard_normal((n, n)) * np.exp2(rng.integers(-300, 300, (n, n)).astype(np.float64))
    a.ravel()[:: 7] = 0.0
    a.ravel()[3:: 11] = -0.0
    a.ravel()[5:: 13] = rng.standard_normal(a.ravel()[5:: 13].shape) * 1e6  # the common range
    want = exact_norm(a, r)
    assert abs(device_norm(cuda, a, r) - want) <= REL_TOL * want


@pytest.mark.parametrize("scale", [1.0, 2.0 ** -59, 2.0 ** -61, 2.0 ** 76, 2.0 ** 78])
def test_range_edges(cuda, scale):
    """Values at the edges of the float-pair range ([2^-60, 2^77)) and just outside it."""
    rng = np.random.default_rng(5)
    n, r = 600, 2
    a = (1.0 + rng.random((n, n))) * scale
    want = exact_norm(a, r)
    assert abs(device_norm(cuda, a, r) - want) <= REL_TOL * want


def test_full_significands(cuda):
    """Values whose 53-bit significands are all ones or carry at the rounding bit of the low float."""
    n, r = 512, 1
    rng = np.random.default_rng(9)
    base = np.float64(2.0) - np.ldexp(1.0, -52)  # 1.111...1 (53 ones)
    a = base * np.exp2(rng.integers(-40, 40, (n, n)).astype(np.float64))
    a[::2] = np.nextafter(a[::2], np.inf)
    want = exact_norm(a, r)
    assert abs(device_norm(cuda, a, r) - want) <= REL_TOL * want


def test_specials_propagate(cuda):
    n, r = 64, 2
    a = np.ones((n, n))
    a[10, 10] = np.inf
    assert device_norm(cuda, a, r) == np.inf
    a[10, 10] = np.nan
    assert np.isnan(device_norm(cuda, a, r))
    a[10, 10] = 1.0
    a[0, 0] = np.nan  # outside the interior: not part of the norm
    assert device_norm(cuda, a, r) == 1.0


def test_prk_field_norm_n16384(cuda):
    """PRK's field after one application at the headline size: the analytic value 2 exactly."""
    n, r = 16384, 2
    in_a, in_b, out = kg.alloc(n)
    kg.init(in_a, out)
    kg.apply(kg.STAR, r, in_a, out, in_next=in_b)
    assert abs(kg.norm(r, out) - 2.0) <= 1e-8


def test_dadd_probe_measures_a_plausible_rate(cuda):
    """The binary64 add rate the bench and the sweep divide by: positive and below the SM count
    times a generous 4 adds per SM per clock at 2.5 GHz."""
    rate = kg.probe_dadd()
    sms = cuda.cuda.get_device_properties(0).multi_processor_count
    assert 1e10 < rate < sms * 4 * 2.5e9
