"""The nstream and transpose restatements against the reference's own validation formulas
(Cxx11/nstream-cuda.cu:188-209, Cxx11/transpose-cuda.cu:262-282): they pin the oracle the GPU
parity tests compare with. A planted error must be caught."""
import numpy as np
import pytest

from oracle import prk_neighbours as nb


@pytest.mark.parametrize("length,iterations", [(1, 0), (1001, 10), (65536, 3)])
def test_nstream_matches_reference_checksum(length, iterations):
    A, B, C = np.zeros(length), np.full(length, 2.0), np.full(length, 2.0)
    for _ in range(iterations + 1):
        nb.nstream(A, B, C, 3.0)
    assert nb.nstream_validates(A, iterations)
    A[length // 2] += 1.0  # a planted error
    assert not nb.nstream_validates(A, iterations)


@pytest.mark.parametrize("order,iterations", [(1, 0), (37, 5), (256, 10)])
def test_transpose_matches_reference_formula(order, iterations):
    A, B = nb.transpose_init(order)
    for _ in range(iterations + 1):
        nb.transpose(A, B)
    assert nb.transpose_abserr(B, iterations) < 1e-8
    B[0, order - 1] += 0.5
    assert nb.transpose_abserr(B, iterations) >= 0.5


def test_nstream_rounds_each_operation():
    """The restatement rounds scalar*C, then B + that, then A + that (no fused multiply-add)."""
    A = np.array([1.0]); B = np.array([2.0 ** -53]); C = np.array([1.0 + 2.0 ** -52])
    nb.nstream(A, B, C, 1.0 + 2.0 ** -52)
    s = (1.0 + 2.0 ** -52) * (1.0 + 2.0 ** -52)  # rounded product
    assert A[0] == 1.0 + (2.0 ** -53 + s)


def _sha(a) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def _golden():
    import json
    from pathlib import Path
    return json.loads((Path(__file__).resolve().parent / "golden" / "neighbours_golden.json").read_text())


def test_oracle_reproduces_reference_nstream_arrays():
    """The reference's own nstream driver (Cxx11/nstream.cc, run by tests/golden/make_neighbours_golden.py)
    left these arrays; the restatement reproduces them bit for bit."""
    for c in _golden()["nstream"]:
        assert c["verdict"] == "Solution validates"
        A, B, C = np.zeros(c["length"]), np.full(c["length"], 2.0), np.full(c["length"], 2.0)
        for _ in range(c["iterations"] + 1):
            nb.nstream(A, B, C, 3.0)
        assert (_sha(A), _sha(B), _sha(C)) == (c["A_sha256"], c["B_sha256"], c["C_sha256"]), c


def test_oracle_reproduces_reference_transpose_arrays():
    """Cxx11/transpose.cc's final A and B (tiled and untiled loops), bit for bit. The reference fills
    A row-major with 0 .. order^2-1, which is transpose_init's A[j][i] = order*j + i."""
    for c in _golden()["transpose"]:
        assert c["verdict"] == "Solution validates"
        A, B = nb.transpose_init(c["order"])
        for _ in range(c["iterations"] + 1):
            nb.transpose(A, B)
        assert (_sha(A), _sha(B)) == (c["A_sha256"], c["B_sha256"]), c
