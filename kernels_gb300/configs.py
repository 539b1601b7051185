"""Run the stencil's measurement configurations beyond the headline one and print one JSON line per
case. The cases are seeded synthetic PRK fields (in = i+j, out = 0), the same shapes as:

  sweep   star and grid, R = 1..5, n = 32768, 50 iterations, FP64 and FP32C (tuned depth each, or
          the TMA kernel at --depth D without tuning; --depth 0: every timed application in one
          launch):
          PRK GFLOP/s, algorithmic HBM GB/s and its fraction of the measured peak, the norm check,
          and the FP32C relative error against the FP64 result (bit-identical to the reference's)
  large   star R=4, FP32C at n = 65536 and FP64 at n = 46000, 200 iterations, tuned depth
  batch   the seeded 256-grid batch (kernels_gb300.workloads), FP64 and FP32C, one CUDA graph, tuned
          depth per grid (or --depth D for every grid)
  neighbours  nstream (length n*n = 2^28, the reference's A = 0, B = C = 2, scalar 3) and transpose
          (order n = 16384, A[j][i] = order*j + i, B = 0), 20 timed iterations after one untimed:
          HBM GB/s as the reference rates them (32 B per element and iteration for both) and its
          fraction of the measured peak; validation by the reference's own formulas, on the GPU

  python -m kernels_gb300.configs sweep|large|batch [--n N] [--iterations K] [--radii 1,2,...] [--depth D]
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

import kernels_gb300 as kg

ROOT = Path(__file__).resolve().parents[1]


def peak_gbs() -> float:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"])
    except Exception:
        return 6800.0


def algorithmic_bytes(n: int, r: int, dtype: int) -> float:
    return (16.0 if dtype == kg.FP64 else 8.0) * n * n + 16.0 * (n - 2 * r) ** 2


def sample_points(n: int, r: int, count: int = 256, seed: int = 9):
    rng = np.random.default_rng(seed)
    return [(int(i), int(j)) for i, j in rng.integers(r, n - r, (count, 2))]


def launches_per_run(iterations: int, depth: int) -> int:
    """Launches prk_gb300_run makes for `iterations` timed applications at temporal depth `depth`
    (0: the whole run in one launch); a remainder goes in launches of decreasing powers of two."""
    if depth == 0:
        return 1
    return iterations // depth + bin(iterations % depth).count("1")


def binary64_adds_per_point(pattern: int, r: int, depth: int = 1) -> int:
    """Rounded binary64 adds one FP64 application issues per interior point on whole-number tiles, in
    launches of `depth` applications: for the stencils whose weights are not powers of two, the part
    of the reference's chain the table route leaves on the binary64 pipe plus the add into out
    (prk_gb300_route_split); the power-of-two stencils need none on the certified routes, where the
    sum is exact."""
    split = kg.route_split(pattern, r, depth)
    return 0 if split is None else split[1]


def one_case(torch, pattern: int, r: int, n: int, iterations: int, dtype: int, pts, depth: int | None = None):
    """A PRK run with the tuned kernel and depth (or the TMA kernel at a fixed depth, untuned);
    returns (record, sampled out values)."""
    in_a, in_b, out = kg.alloc(n, dtype)
    kg.init(in_a, out)
    if depth is None:
        tuning = kg.tune(pattern, r, n, dtype)
    else:
        tuning = {"depth": depth, "kernel": "whole" if depth == 0 else "fixed", "tile_rows": 32,
                  "tile_cols": 0, "cols_per_thread": 0}
    t0 = time.perf_counter()
    if depth is None:
        res = kg.run(pattern, r, iterations, in_a, in_b, out, tuned=True)
    else:
        res = kg.run(pattern, r, iterations, in_a, in_b, out, depth=depth or 1, whole=depth == 0)
    wall = time.perf_counter() - t0
    nrm = kg.norm(r, out)
    idx = torch.tensor([i * n + j for i, j in pts], device="cuda")
    if dtype == kg.FP64:
        vals = out.reshape(-1)[idx].cpu().numpy()
    else:
        o2 = out.reshape(-1, 2)[idx].double().cpu().numpy()
        vals = o2[:, 0] + o2[:, 1]
    per_app = res.elapsed_s / iterations
    # HBM: every launch reads in and out once and writes in_next and out once, whatever its depth,
    # so the algorithmic bytes of one launch are those of one application; the fraction of the
    # copy peak is bytes per launch over the launch's time.
    d = tuning["depth"] if tuning["kernel"] != "generic" else 1
    nl = launches_per_run(iterations, d)
    launch_gbs = algorithmic_bytes(n, r, dtype) * nl / res.elapsed_s / 1e9
    rec = {"pattern": "star" if pattern == kg.STAR else "grid", "radius": r, "n": n, "iterations": iterations,
           "dtype": "fp64" if dtype == kg.FP64 else "fp32c",
           "gflops": round(kg.flops(pattern, r, n) / per_app / 1e9, 3),
           "ms_per_application": round(per_app * 1e3, 4), "launches": nl,
           "roofline": {"bound": "hbm" if nl == iterations else "on-chip",
                        "hbm_gbs_per_launch": round(launch_gbs, 1),
                        "frac_of_hbm_peak": round(launch_gbs / peak_gbs(), 4),
                        "note": "algorithmic bytes of one application per launch over launch time"
                                + ("" if nl == iterations else
                                   f"; {iterations // nl if nl else iterations} applications per launch run "
                                   "from shared memory, bound on chip (FP64: shared-memory wavefronts or the "
                                   "binary64 adds; FP32C: the FP32 pipe)")},
           "norm": nrm, "norm_ok": abs(nrm - 2.0 * (iterations + 1)) <= 1e-8,
           "tuning": {k: tuning[k] for k in ("depth", "kernel", "tile_rows", "tile_cols", "cols_per_thread")},
           "wall_s": round(wall, 3)}
    launch_depth = 1 if d == 1 else max(2, iterations // nl)  # d = 0: the whole run in one launch
    adds = binary64_adds_per_point(pattern, r, launch_depth) if dtype == kg.FP64 else 0
    if adds:
        rate = dadd_rate()
        t_adds = adds * (n - 2 * r) ** 2 / rate
        rec["roofline"]["binary64_add_ceiling"] = {
            "adds_per_point": adds, "fixed_point_adds_per_point": kg.route_split(pattern, r, launch_depth)[0],
            "measured_adds_per_s": round(rate, 1),
            "ms_per_application": round(t_adds * 1e3, 4), "frac": round(t_adds / per_app, 4)}
    del in_a, in_b, out, res
    torch.cuda.empty_cache()
    return rec, vals


_DADD: list[float] = []


def dadd_rate() -> float:
    """The device's binary64 add rate, measured once per process (prk_gb300_probe_dadd)."""
    if not _DADD:
        _DADD.append(kg.probe_dadd())
    return _DADD[0]


def run_pair(torch, pattern, r, n64, n32, iterations, depth=None):
    pts64 = sample_points(n64, r)
    rec64, v64 = one_case(torch, pattern, r, n64, iterations, kg.FP64, pts64, depth)
    print(json.dumps(rec64), flush=True)
    pts32 = sample_points(n32, r)
    rec32, v32 = one_case(torch, pattern, r, n32, iterations, kg.FP32C, pts32, depth)
    if n32 != n64:
        # the FP64 values at the FP32C run's own size (the FP64 path is bit-identical to the
        # reference's strict order, which the parity tests check at this size too)
        _, v64 = one_case(torch, pattern, r, n32, iterations, kg.FP64, pts32, depth)
    rec32["rel_err_vs_fp64"] = float(np.max(np.abs(v32 - v64) / np.abs(v64)))
    rec32["rel_err_points"] = len(pts32)
    print(json.dumps(rec32), flush=True)


def run_batch(torch, iterations: int, depth: int | None, count: int):
    from kernels_gb300.workloads import batch_specs
    specs = batch_specs(count)
    for name, dt in (("fp64", kg.FP64), ("fp32c", kg.FP32C)):
        grids = []
        for p, r, n in specs:
            a, b, o = kg.alloc(n, dt)
            kg.init(a, o)
            grids.append((p, r, a, b, o))
        bt = kg.Batch(grids, depth=depth, tuned=depth is None)
        bt.run(iterations, graph=True)  # tuning, capture, warm-up
        for p, r, a, b, o in grids:
            kg.init(a, o)
        t = bt.run(iterations, graph=True)
        norms = bt.norms()
        fl = sum(kg.flops(p, r, n) for p, r, n in specs) * iterations
        print(json.dumps({"config": "batch", "grids": len(specs), "dtype": name, "iterations": iterations,
                          "depth": depth or "tuned", "gflops": round(fl / t / 1e9, 3), "seconds": round(t, 5),
                          "launches": bt.launches(iterations),
                          "norms_ok": all(abs(x - 2.0 * (iterations + 1)) <= 1e-8 for x in norms)}), flush=True)
        bt.close()
        del grids
        torch.cuda.empty_cache()


def run_neighbours(torch, iterations: int, n: int) -> None:
    """nstream (length n*n) and transpose (order n) timed with CUDA events; validated on the device."""
    k = iterations
    length = n * n
    A = torch.zeros(length, dtype=torch.float64, device="cuda")
    B = torch.full((length,), 2.0, dtype=torch.float64, device="cuda")
    C = torch.full((length,), 2.0, dtype=torch.float64, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kg.nstream(A, B, C, scalar=3.0)  # iteration 0, untimed
    e0.record()
    for _ in range(k):
        kg.nstream(A, B, C, scalar=3.0)
    e1.record()
    e1.synchronize()
    t = e0.elapsed_time(e1) * 1e-3 / k
    ar = length * sum(2.0 + 3.0 * 2.0 for _ in range(k + 1))
    asum = float(A.abs().sum())
    gbs = 32.0 * length / t / 1e9
    print(json.dumps({"kernel": "nstream", "length": length, "iterations": k, "ms_per_iteration": round(t * 1e3, 4),
                      "hbm_gbs": round(gbs, 1), "roofline_frac": round(gbs / peak_gbs(), 4),
                      "validates": abs(ar - asum) / asum <= 1e-8}), flush=True)
    del A, B, C
    torch.cuda.empty_cache()
    order = n
    idx = torch.arange(order, dtype=torch.float64, device="cuda")
    A = (order * idx[:, None] + idx[None, :]).contiguous()
    B = torch.zeros((order, order), dtype=torch.float64, device="cuda")
    kg.transpose(A, B)  # iteration 0, untimed
    e0.record()
    for _ in range(k):
        kg.transpose(A, B)
    e1.record()
    e1.synchronize()
    t = e0.elapsed_time(e1) * 1e-3 / k
    ref = (order * idx[None, :] + idx[:, None]) * (1.0 + k) + (k + 1.0) * (k / 2.0)  # B[j][i] = (i*order+j)(K+1)+...
    abserr = float((B - ref).abs().sum())
    gbs = 32.0 * order * order / t / 1e9
    print(json.dumps({"kernel": "transpose", "order": order, "iterations": k, "ms_per_iteration": round(t * 1e3, 4),
                      "hbm_gbs": round(gbs, 1), "roofline_frac": round(gbs / peak_gbs(), 4),
                      "abserr": abserr, "validates": abserr < 1e-8}), flush=True)


def main() -> None:
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("which", choices=["sweep", "large", "batch", "neighbours"])
    ap.add_argument("--depth", type=int, default=None)
    ap.add_argument("--grids", type=int, default=256)
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--iterations", type=int, default=None)
    ap.add_argument("--radii", default="1,2,3,4,5")
    ap.add_argument("--patterns", default="star,grid")
    args = ap.parse_args()
    if args.which == "sweep":
        n = args.n or 32768
        k = args.iterations or 50
        for name in args.patterns.split(","):
            for r in (int(x) for x in args.radii.split(",")):
                run_pair(torch, kg.pattern_of(name), r, n, n, k, args.depth)
    elif args.which == "large":
        k = args.iterations or 200
        run_pair(torch, kg.STAR, 4, args.n or 46000, 65536, k)
    elif args.which == "neighbours":
        run_neighbours(torch, args.iterations or 20, args.n or 16384)
    else:
        run_batch(torch, args.iterations or 50, args.depth, args.grids)


if __name__ == "__main__":
    main()
