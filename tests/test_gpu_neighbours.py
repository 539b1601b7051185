"""nstream and transpose on the GPU against the CPU restatement (oracle/prk_neighbours.py): bit for
bit on random data, the reference's own validation on its initial data, ragged and unaligned
sizes, and the argument checks."""
import numpy as np
import pytest

import kernels_gb300 as kg
from oracle import prk_neighbours as nb

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


@pytest.mark.parametrize("length", [1, 2, 3, 255, 1001, (1 << 20) + 3])
@pytest.mark.parametrize("offsets", [(0, 0, 0), (1, 1, 1), (1, 0, 1), (0, 1, 0)])
def test_nstream_bit_exact(cuda, length, offsets):
    """Random values; A, B, C offset by one element each (16-byte vectors only when they share
    their alignment)."""
    rng = np.random.default_rng(length + 7 * sum(offsets))
    a, b, c = (rng.standard_normal(length) * np.exp2(rng.integers(-20, 20, length)) for _ in range(3))
    scalar = float(rng.standard_normal())
    dev = []
    for v, off in zip((a, b, c), offsets):
        t = cuda.empty(length + 1, dtype=cuda.float64, device="cuda")
        t[off:off + length] = cuda.from_numpy(v)
        dev.append(t[off:off + length])
    want = a.copy()
    for _ in range(3):
        kg.nstream(*dev, scalar=scalar)
        nb.nstream(want, b, c, scalar)
    assert np.array_equal(bits(dev[0].cpu().numpy()), bits(want))
    assert np.array_equal(dev[1].cpu().numpy(), b) and np.array_equal(dev[2].cpu().numpy(), c)


def _mixed(rng, n, bound):
    """Whole numbers up to about `bound` (both signs, both zeros) mixed with fractional values."""
    v = rng.integers(-bound, bound, n).astype(np.float64)
    v[rng.random(n) < 0.05] = 0.0
    v[rng.random(n) < 0.05] = -0.0
    frac = rng.random(n) < 0.1
    v[frac] += 0.5
    v[rng.random(n) < 0.02] = 2.0 ** 20  # just above the certified bound
    return v


@pytest.mark.parametrize("scalar", [3.0, -7.0, 0.0, -0.0, 8.0, 9.0, 2.5])
def test_nstream_exact_route_bit_exact(cuda, scalar):
    """Whole-number data near the certified bounds, mixed in a warp with values outside them; whole
    and non-whole scalars."""
    n = (1 << 16) + 5
    rng = np.random.default_rng(int(abs(scalar) * 10) + 3)
    a, b, c = (_mixed(rng, n, 2 ** 19) for _ in range(3))
    A, B, C_ = (cuda.from_numpy(x.copy()).cuda() for x in (a, b, c))
    want = a.copy()
    for _ in range(3):
        kg.nstream(A, B, C_, scalar=scalar)
        nb.nstream(want, b, c, scalar)
    assert np.array_equal(bits(A.cpu().numpy()), bits(want))


def test_transpose_exact_route_bit_exact(cuda):
    order = 777
    rng = np.random.default_rng(11)
    a = _mixed(rng, order * order, 2 ** 50).reshape(order, order)
    b = _mixed(rng, order * order, 2 ** 50).reshape(order, order)
    # A += 1 edges: 2^k - 1 (the carry steps the exponent), powers of two, 2^53 and above, negatives
    edges = [2.0 ** k - 1 for k in range(1, 54)] + [2.0 ** k for k in range(0, 55)] + [-1.0, -2.0 ** 40, -3.5]
    a.flat[:len(edges)] = edges
    A, B = cuda.from_numpy(a.copy()).cuda(), cuda.from_numpy(b.copy()).cuda()
    for _ in range(3):
        kg.transpose(A, B)
        nb.transpose(a, b)
    assert np.array_equal(bits(A.cpu().numpy()), bits(a))
    assert np.array_equal(bits(B.cpu().numpy()), bits(b))


def test_nstream_reference_validation(cuda):
    length, k = 10_000_019, 10
    A = cuda.zeros(length, dtype=cuda.float64, device="cuda")
    B = cuda.full((length,), 2.0, dtype=cuda.float64, device="cuda")
    C = cuda.full((length,), 2.0, dtype=cuda.float64, device="cuda")
    for _ in range(k + 1):
        kg.nstream(A, B, C, scalar=3.0)
    assert nb.nstream_validates(A.cpu().numpy(), k)


@pytest.mark.parametrize("order", [1, 2, 3, 63, 64, 65, 129, 1000, 2048])
def test_transpose_bit_exact(cuda, order):
    rng = np.random.default_rng(order)
    a = rng.standard_normal((order, order)) * np.exp2(rng.integers(-20, 20, (order, order)))
    b = rng.standard_normal((order, order))
    A, B = cuda.from_numpy(a.copy()).cuda(), cuda.from_numpy(b.copy()).cuda()
    for _ in range(2):
        kg.transpose(A, B)
        nb.transpose(a, b)
    assert np.array_equal(bits(A.cpu().numpy()), bits(a))
    assert np.array_equal(bits(B.cpu().numpy()), bits(b))


@pytest.mark.parametrize("order,k", [(1024, 10), (4096, 5), (999, 7)])
def test_transpose_reference_validation(cuda, order, k):
    a, b = nb.transpose_init(order)
    A, B = cuda.from_numpy(a).cuda(), cuda.from_numpy(b).cuda()
    for _ in range(k + 1):
        kg.transpose(A, B)
    assert nb.transpose_abserr(B.cpu().numpy(), k) < 1e-8
    assert np.array_equal(A.cpu().numpy(), a + k + 1)


def test_neighbour_rejections(cuda):
    lib = kg.load()
    A = cuda.zeros(1024, dtype=cuda.float64, device="cuda")
    assert lib.prk_gb300_nstream(0, 3.0, A.data_ptr(), A.data_ptr(), A.data_ptr(), None) == -1
    assert lib.prk_gb300_nstream(512, 3.0, A.data_ptr(), A[256:].data_ptr(), A[600:].data_ptr(), None) == -1  # A overlaps B
    assert lib.prk_gb300_nstream(16, 3.0, None, A.data_ptr(), A.data_ptr(), None) == -1
    M = cuda.zeros((32, 32), dtype=cuda.float64, device="cuda")
    assert lib.prk_gb300_transpose(32, M.data_ptr(), M.data_ptr(), None) == -1  # A is B
    assert lib.prk_gb300_transpose(0, M.data_ptr(), M.data_ptr(), None) == -1
    assert lib.prk_gb300_transpose(1 << 23, M.data_ptr(), None, None) == -1


def _sha(a) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def test_gpu_reproduces_reference_driver_arrays(cuda):
    """The arrays the reference's own nstream and transpose drivers (Cxx11/nstream.cc,
    Cxx11/transpose.cc) left after their runs (tests/golden/neighbours_golden.json), bit for bit."""
    import json
    from pathlib import Path
    g = json.loads((Path(__file__).resolve().parent / "golden" / "neighbours_golden.json").read_text())
    for c in g["nstream"]:
        n = c["length"]
        A = cuda.zeros(n, dtype=cuda.float64, device="cuda")
        B = cuda.full((n,), 2.0, dtype=cuda.float64, device="cuda")
        C = cuda.full((n,), 2.0, dtype=cuda.float64, device="cuda")
        for _ in range(c["iterations"] + 1):
            kg.nstream(A, B, C, scalar=3.0)
        assert (_sha(A.cpu().numpy()), _sha(B.cpu().numpy()), _sha(C.cpu().numpy())) == \
            (c["A_sha256"], c["B_sha256"], c["C_sha256"]), c
    for c in g["transpose"]:
        a, b = nb.transpose_init(c["order"])
        A, B = cuda.from_numpy(a).cuda(), cuda.from_numpy(b).cuda()
        for _ in range(c["iterations"] + 1):
            kg.transpose(A, B)
        assert (_sha(A.cpu().numpy()), _sha(B.cpu().numpy())) == (c["A_sha256"], c["B_sha256"]), c
