"""Parity of the CUDA path (through the C ABI) with the oracle and the reference's golden outputs.

FP64: bit-identical to the reference's strict-order binary64 evaluation, on the reference's CI
matrix, tiny and odd sizes, random non-integer fields, and sampled points at n=16384.
FP32C: relative error of hi+lo against the FP64 oracle at most 1e-6 (the bound the stencil's
compensated form is specified to), and the PRK norm check.
"""
import hashlib

import numpy as np
import pytest

import kernels_gb300 as kg
from oracle import prk_oracle as po

pytestmark = pytest.mark.gpu

PAT = {"star": kg.STAR, "grid": kg.GRID}
FP32C_REL_TOL = 1e-6


def device_run(torch, pattern, r, n, iterations, dtype=kg.FP64, graph=False, unfused=False):
    in_a, in_b, out = kg.alloc(n, dtype, ping_pong=not unfused)
    kg.init(in_a, out)
    res = kg.run(pattern, r, iterations, in_a, in_b, out, graph=graph, unfused=unfused)
    torch.cuda.synchronize()
    return res, out


def out_as_f64(out) -> np.ndarray:
    a = out.cpu().numpy()
    if a.dtype == np.float32:
        return a[..., 0].astype(np.float64) + a[..., 1].astype(np.float64)
    return a


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(a.astype("<f8").tobytes()).hexdigest()


@pytest.mark.parametrize("idx", range(11))
@pytest.mark.parametrize("mode", ["fused", "graph", "unfused"])
def test_ci_matrix_fp64_bit_exact(cuda, golden, idx, mode):
    c = golden["cases"][idx]
    res, out = device_run(cuda, PAT[c["pattern"]], c["radius"], c["n"], c["iterations"],
                          graph=mode == "graph", unfused=mode == "unfused")
    got = out_as_f64(out)
    assert sha(got) == c["out_sha256"]
    n = c["n"]
    fin = res.final_in.cpu().numpy()
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    assert np.array_equal(fin, (ii + jj + c["iterations"] + 1).astype(np.float64))
    nrm = kg.norm(c["radius"], out)
    assert abs(nrm - float.fromhex(c["norm_hex"])) <= 1e-13 * nrm
    assert abs(nrm - 2.0 * (c["iterations"] + 1)) <= 1e-8


def test_reference_operator_names(cuda, golden):
    """star1..5/grid1..5(n, t, in, out) update out only, exactly like the reference operator."""
    c = golden["cases"][3]  # star 3, n=200
    n = c["n"]
    in_ = cuda.empty((n, n), dtype=cuda.float64, device="cuda")
    out = cuda.empty((n, n), dtype=cuda.float64, device="cuda")
    kg.init(in_, out)
    before = in_.clone()
    for _ in range(c["iterations"] + 1):
        kg.star3(n, c["tile"], in_, out)
        kg.add(in_)
    assert sha(out.cpu().numpy()) == c["out_sha256"]
    assert cuda.equal(in_, before + (c["iterations"] + 1))


def test_tiny_and_odd_sizes_fp64(cuda, golden, tiny_arrays):
    for c in golden["tiny"]:
        _, out = device_run(cuda, PAT[c["pattern"]], c["radius"], c["n"], c["iterations"])
        ref = tiny_arrays[c["key"]]
        assert np.array_equal(out.cpu().numpy().view(np.uint64), ref.view(np.uint64)), c["key"]


@pytest.mark.parametrize("pattern", [kg.STAR, kg.GRID])
@pytest.mark.parametrize("r", range(1, 6))
@pytest.mark.parametrize("n", [61, 256, 515])
def test_random_fields_fp64_bit_exact(cuda, pattern, r, n):
    """Arbitrary (non-integer, mixed-sign, mixed-exponent) fields: one fused application."""
    rng = np.random.default_rng(1000 * pattern + 10 * r + n)
    a = rng.standard_normal((n, n)) * np.exp2(rng.integers(-20, 20, (n, n)))
    o = rng.standard_normal((n, n)) * 100.0
    in_ = cuda.from_numpy(a).cuda()
    out = cuda.from_numpy(o.copy()).cuda()
    nxt = cuda.empty_like(in_)
    kg.apply(pattern, r, in_, out, in_next=nxt)
    cuda.cuda.synchronize()
    po.apply(pattern, r, a, o)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), o.view(np.uint64))
    assert np.array_equal(nxt.cpu().numpy().view(np.uint64), (a + 1.0).view(np.uint64))


@pytest.mark.parametrize("idx", range(11))
def test_ci_matrix_fp32c_error_bound(cuda, golden, idx):
    c = golden["cases"][idx]
    r, n = c["radius"], c["n"]
    _, out = device_run(cuda, PAT[c["pattern"]], r, n, c["iterations"], dtype=kg.FP32C)
    _, ref = po.run(PAT[c["pattern"]], r, n, c["iterations"], c["tile"])
    got = out_as_f64(out)
    inner = (slice(r, n - r), slice(r, n - r))
    rel = np.abs(got[inner] - ref[inner]) / np.abs(ref[inner])
    assert rel.max() <= FP32C_REL_TOL
    assert np.all(got[:r] == 0) and np.all(got[n - r:] == 0)
    nrm = kg.norm(r, out)
    assert abs(nrm - 2.0 * (c["iterations"] + 1)) <= 1e-8


@pytest.mark.parametrize("pattern", ["star", "grid"])
def test_full_size_n16384_properties(cuda, pattern):
    """The headline workload: n=16384, 100 iterations, FP64. Norm check, sampled points against
    the per-point oracle (bit-exact), and the final `in` field."""
    n, K, r = 16384, 100, 2
    res, out = device_run(cuda, PAT[pattern], r, n, K)
    nrm = kg.norm(r, out)
    assert abs(nrm - 2.0 * (K + 1)) <= 1e-8
    rng = np.random.default_rng(7)
    pts = [(r, r), (n - r - 1, n - r - 1), (r, n - r - 1), (8191, 8192)] + \
          [tuple(int(x) for x in rng.integers(r, n - r, 2)) for _ in range(60)]
    idx = cuda.tensor([i * n + j for i, j in pts], device="cuda")
    got = out.reshape(-1)[idx].cpu().numpy()
    for (i, j), v in zip(pts, got):
        assert v == po.point(PAT[pattern], r, n, K + 1, i, j), (i, j)
    fin = res.final_in.reshape(-1)[idx].cpu().numpy()
    assert all(f == i + j + K + 1 for (i, j), f in zip(pts, fin))


def test_run_host_matches_device_run(cuda, golden):
    c = golden["cases"][0]  # star 2, n=1000
    n = c["n"]
    h_in = np.add.outer(np.arange(n), np.arange(n)).astype(np.float64)
    h_out = np.zeros((n, n))
    h_fin = np.empty_like(h_in)
    res = kg.run_host(kg.STAR, 2, c["iterations"], h_in, h_out, h_fin)
    assert sha(h_out) == c["out_sha256"]
    assert np.array_equal(h_fin, h_in + c["iterations"] + 1)
    assert abs(res["norm"] - 22.0) <= 1e-8
    assert res["elapsed_s"] > 0 and res["kernel_s"] > 0


def test_rejected_calls_raise(cuda):
    in_a, in_b, out = kg.alloc(64)
    with pytest.raises(kg.PrkError) as e:
        kg.run(kg.STAR, 6, 3, in_a, in_b, out)
    assert e.value.code == -1
    with pytest.raises(kg.PrkError):
        kg.run(kg.STAR, 2, 0, in_a, in_b, out)
    with pytest.raises(kg.PrkError):
        kg.apply(kg.STAR, 2, in_a, out, in_next=in_a)  # in_next overlaps in
    small = kg.alloc(4)
    with pytest.raises(kg.PrkError):
        kg.apply(kg.GRID, 2, small[0], small[2])  # 2R+1 > n


def test_bounded_wait_reports_timeout_and_gpu_stays_usable(cuda):
    """A kernel waits on an mbarrier nobody arrives on; its bounded wait gives up, the status word
    turns into PRK_ERR_TIMEOUT, and the next stencil call still works."""
    from kernels_gb300 import _lib
    lib = _lib.load()
    assert lib.prk_gb300_selftest_timeout() == -4
    assert b"gave up" in lib.prk_gb300_last_error()
    kg.status()  # cleared
    n = 64
    in_a, in_b, out = kg.alloc(n)
    kg.init(in_a, out)
    kg.run(kg.STAR, 2, 3, in_a, in_b, out)
    assert abs(kg.norm(2, out) - 8.0) <= 1e-8


@pytest.mark.parametrize("args", [("10", "1000"), ("10", "200", "20", "grid", "3"), ("10", "200", "20", "star", "5", "--unfused"),
                                  ("10", "1000", "32", "star", "2", "--dtype", "fp32c", "--graph"),
                                  ("10", "1000", "32", "grid", "2", "--whole"), ("10", "1000", "32", "star", "2", "--tuned"),
                                  ("10", "1000", "32", "star", "3", "--dtype", "fp32c", "--whole", "--graph")])
def test_cli_driver_validates(cuda, args):
    """The C++ driver with the reference CLI prints the reference's verdict and rate lines."""
    import subprocess
    from pathlib import Path
    cli = Path(__file__).resolve().parents[1] / "kernels_gb300" / "_build" / "stencil-gb300"
    res = subprocess.run([str(cli), *args], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "Solution validates" in res.stdout
    assert "Rate (MFlops/s): " in res.stdout and "Avg time (s): " in res.stdout
    assert "L1 norm = 22 Reference L1 norm = 22" in res.stdout
