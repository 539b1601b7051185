"""The reference's own CUDA stencil beside this library's kernels on the same GPU.

oracle/_ref/stencil_cuda.cubin is Cxx11/stencil-cuda.cu's device code compiled for sm_103a from the
reference sources (make -C oracle ref-cuda); oracle/ref_cuda.py drives it the way stencil-cuda.cu
does. The results agree within 1e-12 relative: nvcc contracts the reference's products and sums
into FMAs, so its rounding is not the strict left-to-right order the FP64 path reproduces. The last
test measures both on the headline configuration and prints one JSON line with the speed-up."""
import json

import numpy as np
import pytest

import kernels_gb300 as kg
from oracle import ref_cuda

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_cuda.available(),
                                 reason="oracle/_ref/stencil_cuda.cubin is not built (make -C oracle ref-cuda)")]

CI = [(p, r) for p in ("star", "grid") for r in range(1, 6)]


def reference_run(torch, pattern, r, n, k, tile):
    idx = torch.arange(n, dtype=torch.float64, device="cuda")
    d_in = (idx[:, None] + idx[None, :]).contiguous()
    d_out = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    seconds = ref_cuda.run(pattern, r, n, k, d_in.data_ptr(), d_out.data_ptr(), tile)
    return d_in, d_out, seconds


@pytest.mark.parametrize("pattern,r", CI)
def test_reference_cuda_agrees(cuda, pattern, r):
    """The reference's CI cases (ci/build-run-prk.sh: 10 iterations, n=200, tile 20)."""
    n, k, tile = 200, 10, 20
    d_in, d_out, _ = reference_run(cuda, pattern, r, n, k, tile)
    in_a, in_b, out = kg.alloc(n, kg.FP64)
    kg.init(in_a, out)
    kg.run(kg.pattern_of(pattern), r, k, in_a, in_b, out)
    ours, theirs = out.cpu().numpy(), d_out.cpu().numpy()
    inner = (slice(r, n - r), slice(r, n - r))
    assert np.abs(theirs[inner] - ours[inner]).max() <= 1e-12 * np.abs(ours[inner]).max()
    assert np.array_equal(theirs[:r], ours[:r]) and not theirs[:r].any()  # boundary rows untouched
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    assert np.array_equal(d_in.cpu().numpy(), (ii + jj + k + 1).astype(np.float64))
    assert abs(kg.norm(r, d_out) - 2.0 * (k + 1)) <= 1e-8


def test_speedup_over_reference_cuda(cuda):
    """star R=2, n=16384: the reference's loop (stencil kernel, add kernel, device synchronise per
    iteration, tile 32) against the fused TMA kernel, one application per launch, and against the
    whole run in one launch per tile."""
    pattern, r, n, k = "star", 2, 16384, 20
    d_in, d_out, t_ref = reference_run(cuda, pattern, r, n, k, 32)
    nrm_ref = kg.norm(r, d_out)
    sample = d_out[4096:4100, 8192:8196].cpu().numpy()
    del d_in, d_out
    cuda.cuda.empty_cache()
    in_a, in_b, out = kg.alloc(n, kg.FP64)
    kg.init(in_a, out)
    t_ours = kg.run(kg.STAR, r, k, in_a, in_b, out).elapsed_s
    assert abs(kg.norm(r, out) - nrm_ref) <= 1e-8
    assert np.abs(out[4096:4100, 8192:8196].cpu().numpy() - sample).max() <= 1e-12 * np.abs(sample).max()
    kg.init(in_a, out)
    t_whole = kg.run(kg.STAR, r, k, in_a, in_b, out, whole=True).elapsed_s
    fl = kg.flops(kg.STAR, r, n) * k
    rec = {"comparator": "reference Cxx11/stencil-cuda.cu (sm_103a), star R=2 n=16384, 20 timed iterations",
           "reference_ms_per_iteration": round(t_ref / k * 1e3, 4),
           "reference_gflops": round(fl / t_ref / 1e9, 3),
           "fused_ms_per_iteration": round(t_ours / k * 1e3, 4),
           "fused_gflops": round(fl / t_ours / 1e9, 3),
           "whole_run_gflops": round(fl / t_whole / 1e9, 3),
           "speedup_fused": round(t_ref / t_ours, 2), "speedup_whole_run": round(t_ref / t_whole, 2)}
    print(json.dumps(rec))
    assert t_ours < t_ref
