"""The oracle against the reference's own outputs (golden fixtures) and the analytic answers."""
import hashlib
from fractions import Fraction

import numpy as np
import pytest

from oracle import prk_oracle as po

PAT = {"star": po.STAR, "grid": po.GRID}


def generator_weights(pattern: str, r: int) -> dict[tuple[int, int], float]:
    """The weight matrix as Cxx11/generate-cxx-stencil.py:209-230 builds it, W[col+R][row+R],
    restated independently of the oracle: returns {(dc, dr): w} for the nonzero taps."""
    W = [[0.0] * (2 * r + 1) for _ in range(2 * r + 1)]
    if pattern == "star":
        for i in range(1, r + 1):
            W[r][r + i] = +1. / (2 * i * r)
            W[r + i][r] = +1. / (2 * i * r)
            W[r][r - i] = -1. / (2 * i * r)
            W[r - i][r] = -1. / (2 * i * r)
    else:
        for j in range(1, r + 1):
            for i in range(-j + 1, j):
                W[r + i][r + j] = +1. / (4 * j * (2 * j - 1) * r)
                W[r + i][r - j] = -1. / (4 * j * (2 * j - 1) * r)
                W[r + j][r + i] = +1. / (4 * j * (2 * j - 1) * r)
                W[r - j][r + i] = -1. / (4 * j * (2 * j - 1) * r)
            W[r + j][r + j] = +1. / (4 * j * r)
            W[r - j][r - j] = -1. / (4 * j * r)
    return {(a - r, b - r): W[a][b] for a in range(2 * r + 1) for b in range(2 * r + 1) if W[a][b] != 0.0}


@pytest.mark.parametrize("pattern", ["star", "grid"])
@pytest.mark.parametrize("r", range(1, 6))
def test_taps_follow_generator(pattern, r):
    want = generator_weights(pattern, r)
    taps = po.taps(PAT[pattern], r)
    # emission order: column offset outer, row offset inner (generate-cxx-stencil.py:15-38)
    assert [(dc, dr) for dc, dr, _ in taps] == sorted(want)
    for dc, dr, w in taps:
        assert w == want[(dc, dr)]  # bit-identical weights
    assert len(taps) == (4 * r if pattern == "star" else 4 * r * r + 2 * r)
    # antisymmetry W[-d] = -W[d], sum w = 0, sum w*d = 1 per axis (so each application adds 2)
    for (dc, dr), w in want.items():
        assert want[(-dc, -dr)] == -w
    exact = {k: Fraction(v) for k, v in want.items()}
    assert sum(exact.values()) == 0
    assert abs(sum(w * dc for (dc, dr), w in exact.items()) - 1) < Fraction(1, 10**12)
    assert abs(sum(w * dr for (dc, dr), w in exact.items()) - 1) < Fraction(1, 10**12)


@pytest.mark.parametrize("idx", range(11))
def test_oracle_matches_reference_run(golden, idx):
    c = golden["cases"][idx]
    _, out = po.run(PAT[c["pattern"]], c["radius"], c["n"], c["iterations"], c["tile"])
    assert hashlib.sha256(out.astype("<f8").tobytes()).hexdigest() == c["out_sha256"]
    assert po.norm(c["radius"], out) == float.fromhex(c["norm_hex"])
    for i, j, v in c["points"]:
        assert out[i, j] == float.fromhex(v)
        # the per-point oracle (no grid) gives the same bits
        assert po.point(PAT[c["pattern"]], c["radius"], c["n"], c["iterations"] + 1, i, j) == float.fromhex(v)


def test_reference_drivers_validate(golden):
    for c in golden["cases"]:
        assert c["ref_stencil"]["validates"] and c["ref_stencil_openmp"]["validates"]
        want = 2.0 * (c["iterations"] + 1)
        assert abs(float.fromhex(c["norm_hex"]) - want) <= 1e-8
        # the reference's own fast-math build stays within 1e-12 absolute of the strict order
        assert c["fastmath_max_abs_diff"] < 1e-12


def test_oracle_tiny_full_arrays(golden, tiny_arrays):
    for c in golden["tiny"]:
        _, out = po.run(PAT[c["pattern"]], c["radius"], c["n"], c["iterations"], c["tile"])
        ref = tiny_arrays[c["key"]]
        assert out.view(np.uint64).tobytes() == ref.astype("<f8").view(np.uint64).tobytes(), c["key"]


def test_oracle_rejects_bad_arguments():
    with pytest.raises(ValueError):
        po.run(po.STAR, 0, 10, 1)
    with pytest.raises(ValueError):
        po.run(po.STAR, 6, 100, 1)
    with pytest.raises(ValueError):
        po.run(po.GRID, 3, 6, 1)  # 2R+1 > n
    with pytest.raises(ValueError):
        po.run(po.STAR, 1, 10, 0)


def test_point_oracle_at_large_n():
    # interior points of n=65536 (beyond the reference's 46340 cap): the analytic value 2*(K+1)
    # holds exactly for the power-of-two stencils and within rounding for the others
    for pattern in (po.STAR, po.GRID):
        for r in range(1, 6):
            v = po.point(pattern, r, 65536, 51, 65536 - r - 1, 40000)
            assert abs(v - 102.0) < 1e-9


def test_flops():
    assert po.flops(po.STAR, 2, 16384) == (2 * 9 + 1) * 16380.0 ** 2
    assert po.flops(po.GRID, 2, 16384) == (2 * 25 + 1) * 16380.0 ** 2
