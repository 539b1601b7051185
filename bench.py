"""Benchmark of the PRK 2D stencil hot path on GB300.

Workload (one "step" = one fused application over the whole grid: out += S(in) on the interior and
in_next = in + 1 everywhere): star R=2, n=16384, FP64 storage, in(i,j)=i+j, out=0 -- the PRK
stencil at 2.1 GB per array, the configuration the headline metric is quoted on. Every array is far
larger than the 129 MB L2, so no flush is needed between steps. The same workload is also measured
in the FP32-compensated form (the "fp32c" key) with its relative error against the FP64 path, whose
results are bit-identical to the reference's (the parity tests check that), and as the seeded
256-grid batched configuration (the "batched" key). The "grid2" key is the grid R=2 stencil on the
same grid, FP64, with both of its ceilings (HBM and the binary64 add rate, measured in the run), and
"gpu_comparator" times the reference's own CUDA stencil (Cxx11/stencil-cuda.cu built for sm_103a)
on the headline grid, outside the timed region, when its cubin was built.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's CPU implementation of the path (the OpenMP stencil, here as
the oracle's port compiled with the reference's flags) on the host cores, same metric and config.
With N > 1 (torchrun), each rank runs an independent replica of the workload (the stencil path has
no exchange step on one grid per GPU); value is the sum over ranks, timed by the slowest rank.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GFLOP/s + HBM GB/s, star R=2 n=16384: FP64 vs FP32-comp (rel err<=1e-6)"
N_DEFAULT, R_DEFAULT = 16384, 2
PEAK_FALLBACK_GBS = 6800.0
L2_BYTES = 129 * 2**20  # GB300's last-level cache, for the config's L2 note


def algorithmic_bytes(n: int, r: int, fp64: bool) -> float:
    """Bytes one fused application must move: in read + in_next write over n^2, out read + write
    over the interior. FP64: 16 n^2 + 16 (n-2R)^2. FP32C: 8 n^2 + 16 (n-2R)^2."""
    return (16.0 if fp64 else 8.0) * n * n + 16.0 * (n - 2 * r) ** 2


def hbm_peak() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return PEAK_FALLBACK_GBS, "fallback"


def profiled_traffic() -> dict:
    """DRAM bytes per launch from the committed ncu capture summary, if present."""
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return {}
    return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        mhz, maxmhz, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                mhz.append(float(f[1]))
                maxmhz = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": maxmhz,
                "reasons": sorted(reasons), "samples": len(mhz)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_port_rate(pattern: int, r: int, n: int, applications: int, threads: int | None = None) -> dict:
    """GFLOP/s of the CPU port (oracle compiled with the reference's -O3 -ffast-math -fopenmp) over
    `applications` applications at size n, on all host cores unless `threads` is given."""
    import numpy as np
    from oracle import prk_oracle as po
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    lib = po.cpu_baseline()
    a = np.empty((n, n))
    o = np.empty((n, n))
    lib.prk_oracle_init(n, 32, a.ctypes.data, o.ctypes.data)
    lib.prk_oracle_sample(pattern, r, n, 1, 32, a.ctypes.data, o.ctypes.data)  # warm-up (first touch)
    t = lib.prk_oracle_sample(pattern, r, n, applications, 32, a.ctypes.data, o.ctypes.data)
    fl = po.flops(pattern, r, n)
    return {"gflops": fl * applications / t / 1e9, "seconds": t, "threads": int(lib.prk_oracle_threads()),
            "gbs": algorithmic_bytes(n, r, True) * applications / t / 1e9}


def run_reference(args) -> None:
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    from oracle import prk_oracle as po
    import numpy as np
    n, r, pattern = args.n, args.radius, 0
    lib = po.cpu_baseline()
    a = np.empty((n, n))
    o = np.empty((n, n))
    lib.prk_oracle_init(n, 32, a.ctypes.data, o.ctypes.data)
    lib.prk_oracle_sample(pattern, r, n, max(args.warmup, 1), 32, a.ctypes.data, o.ctypes.data)
    t = lib.prk_oracle_sample(pattern, r, n, args.steps, 32, a.ctypes.data, o.ctypes.data)
    fl = po.flops(pattern, r, n)
    value = fl * args.steps / t / 1e9
    threads = int(lib.prk_oracle_threads())
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * t / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"PRK star stencil R={r}, n={n}, FP64, one application + in+=1 per step",
                   "pattern": "star", "radius": r, "n": n,
                   "l2": "inputs larger than L2" if 8 * n * n > L2_BYTES else "inputs within L2 (a small case)"},
        "hbm_gbs": round(algorithmic_bytes(n, r, True) * args.steps / t / 1e9, 2),
        "cpu_baseline": {"value": round(value, 3), "unit": "GFLOP/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} applications at n={n} (stencil-openmp loop restated in C, "
                                   f"-O3 -ffast-math -fopenmp, OMP_NUM_THREADS={threads})"},
        "e2e": {"value": round(value, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def reference_cuda_rate(torch, kg, n: int, r: int, iterations: int = 20) -> dict | None:
    """The reference's CUDA stencil (Cxx11/stencil-cuda.cu compiled for sm_103a into
    oracle/_ref/stencil_cuda.cubin) driven as its own loop drives it (stencil kernel, add kernel and
    a device synchronise per iteration, tile 32), star R at size n, beside the fused tile kernel on
    the same grid. A baseline, timed outside this benchmark's timed region; None when the cubin was
    not built."""
    try:
        from oracle import ref_cuda
    except Exception:
        return None
    if not ref_cuda.available():
        return None
    idx = torch.arange(n, dtype=torch.float64, device="cuda")
    d_in = (idx[:, None] + idx[None, :]).contiguous()
    d_out = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    t_ref = ref_cuda.run("star", r, n, iterations, d_in.data_ptr(), d_out.data_ptr(), 32)
    nrm_ref = kg.norm(r, d_out)
    del d_in, d_out, idx
    torch.cuda.empty_cache()
    fl = kg.flops(kg.STAR, r, n) * iterations
    return {"what": f"reference Cxx11/stencil-cuda.cu (device code compiled for sm_103a from the reference "
                    f"sources), star R={r}, n={n}, {iterations} timed iterations, tile 32, its own loop",
            "ms_per_iteration": round(t_ref / iterations * 1e3, 4), "gflops": round(fl / t_ref / 1e9, 3),
            "norm_check": abs(nrm_ref - 2.0 * (iterations + 1)) <= 1e-8}


def time_steps(torch, kg, pattern, r, bufs, out, steps, warmup, stream) -> tuple[float, int]:
    """W untimed + K timed fused applications on `stream`; returns (seconds, final parity)."""
    cur = 0
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            kg.apply(pattern, r, bufs[cur], out, in_next=bufs[cur ^ 1], stream=stream)
            cur ^= 1
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        stream.synchronize()
        e0.record(stream)
        for _ in range(steps):
            kg.apply(pattern, r, bufs[cur], out, in_next=bufs[cur ^ 1], stream=stream)
            cur ^= 1
        e1.record(stream)
        e1.synchronize()
    return e0.elapsed_time(e1) * 1e-3, cur


def time_depth(torch, kg, pattern, r, bufs, out, apps, depth, stream) -> float:
    """`apps` applications as apps/depth launches of `depth` applications each; returns seconds."""
    cur = 0
    with torch.cuda.stream(stream):
        for _ in range(3):  # warm-up launches
            kg.apply_steps(pattern, r, depth, bufs[cur], out, bufs[cur ^ 1], stream=stream)
            cur ^= 1
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        stream.synchronize()
        e0.record(stream)
        for _ in range(apps // depth):
            kg.apply_steps(pattern, r, depth, bufs[cur], out, bufs[cur ^ 1], stream=stream)
            cur ^= 1
        e1.record(stream)
        e1.synchronize()
    return e0.elapsed_time(e1) * 1e-3


def run_gb300(args) -> None:
    import numpy as np
    import torch
    import kernels_gb300 as kg

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    n, r, pattern = args.n, args.radius, kg.STAR
    stream = torch.cuda.Stream()
    fl = kg.flops(pattern, r, n)

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        if not dist:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # ---- FP64 (headline) ----
    in_a, in_b, out = kg.alloc(n, kg.FP64)
    kg.init(in_a, out)
    barrier()
    clocks = ClockSampler(local).__enter__()  # sampled over every timed section below, until the e2e calls end
    t64, cur = time_steps(torch, kg, pattern, r, (in_a, in_b), out, args.steps, args.warmup, stream)
    barrier()
    t64 = max_over_ranks(t64)
    apps = args.steps + args.warmup
    nrm = kg.norm(r, out)
    norm_ok = abs(nrm - 2.0 * apps) <= 1e-8  # apps applications ran: norm = 2 * apps
    # sampled FP64 values (bit-identical to the strict-order reference, as the parity tests show)
    # against which the FP32C form's error is measured
    rng = np.random.default_rng(3)
    pts = [(int(i), int(j)) for i, j in rng.integers(r, n - r, (256, 2))]
    idx = torch.tensor([i * n + j for i, j in pts], device="cuda")
    ref64 = out.reshape(-1)[idx].cpu().numpy()
    temporal = {"fp64": {}, "fp32c": {}}
    if not args.no_temporal:
        for depth in (2, 4, 8):
            td = time_depth(torch, kg, pattern, r, (in_a, in_b), out, 8 * (args.steps // 8 or 1), depth, stream)
            napps = 8 * (args.steps // 8 or 1)
            temporal["fp64"][str(depth)] = round(fl * napps / td / 1e9, 3)
        tw = kg.run(pattern, r, args.steps, in_a, in_b, out, whole=True, stream=stream).elapsed_s
        temporal["fp64"][str(args.steps)] = round(fl * args.steps / tw / 1e9, 3)
    del in_a, in_b, out
    torch.cuda.empty_cache()

    # ---- FP32C (the compensated form) on the same workload ----
    in_a, in_b, out = kg.alloc(n, kg.FP32C)
    kg.init(in_a, out)
    barrier()
    t32, _ = time_steps(torch, kg, pattern, r, (in_a, in_b), out, args.steps, args.warmup, stream)
    barrier()
    t32 = max_over_ranks(t32)
    nrm32 = kg.norm(r, out)
    o2 = out.reshape(-1, 2)[idx].double().cpu().numpy()
    got = o2[:, 0] + o2[:, 1]
    rel32 = float(np.max(np.abs(got - ref64) / np.abs(ref64)))
    if not args.no_temporal:
        for depth in (2, 4, 8):
            napps = 8 * (args.steps // 8 or 1)
            td = time_depth(torch, kg, pattern, r, (in_a, in_b), out, napps, depth, stream)
            temporal["fp32c"][str(depth)] = round(fl * napps / td / 1e9, 3)
        tw = kg.run(pattern, r, args.steps, in_a, in_b, out, whole=True, stream=stream).elapsed_s
        temporal["fp32c"][str(args.steps)] = round(fl * args.steps / tw / 1e9, 3)
    del in_a, in_b, out
    torch.cuda.empty_cache()

    # ---- grid R=2, the other half of the headline configuration, FP64, one application per launch ----
    grid2 = None
    if not args.no_grid:
        in_a, in_b, out = kg.alloc(n, kg.FP64)
        kg.init(in_a, out)
        barrier()
        g_steps = max(args.steps // 4, 5)
        tg, _ = time_steps(torch, kg, kg.GRID, r, (in_a, in_b), out, g_steps, args.warmup, stream)
        barrier()
        tg = max_over_ranks(tg)
        nrm_g = kg.norm(r, out)
        del in_a, in_b, out
        torch.cuda.empty_cache()
        fl_g = kg.flops(kg.GRID, r, n)
        per_g = tg / g_steps
        bg = algorithmic_bytes(n, r, True)
        t_hbm = bg / (hbm_peak()[0] * 1e9)
        rate = kg.probe_dadd()
        # the reference's chain rounds every one of its adds: on whole-number tiles the table route
        # runs the first part of each chain in exact fixed point on the integer pipes and the rest,
        # with the add into out, on the binary64 pipe
        fixed_adds, dp_adds = kg.route_split(kg.GRID, r, 1)  # one application per launch
        pts = (n - 2 * r) ** 2
        t_dadd = dp_adds * pts / rate
        grid2 = {"value": round(world * fl_g / per_g / 1e9, 3), "unit": "GFLOP/s", "steps": g_steps,
                 "ms_per_step": round(per_g * 1e3, 4),
                 "norm_check": abs(nrm_g - 2.0 * (g_steps + args.warmup)) <= 1e-8,
                 "workload": f"PRK grid stencil R={r}, n={n}, FP64, one fused application per step",
                 "roofline": {"bound": "arithmetic (binary64 adds and integer pipes)" if t_dadd > 0.5 * t_hbm else "hbm",
                              "hbm": {"achieved": round(bg / per_g / 1e9, 2), "peak": hbm_peak()[0], "unit": "GB/s",
                                      "frac": round(t_hbm / per_g, 4)},
                              "binary64_adds": {"adds_per_point": dp_adds, "peak_adds_per_s": round(rate, 1),
                                                "achieved_adds_per_s": round(dp_adds * pts / per_g, 1),
                                                "frac": round(t_dadd / per_g, 4),
                                                "peak_source": "prk_gb300_probe_dadd, measured in this run"},
                              "fixed_point_adds": {"adds_per_point": fixed_adds,
                                                   "achieved_adds_per_s": round(fixed_adds * pts / per_g, 1),
                                                   "where": "integer pipes, about 25 integer instructions each"},
                              "note": "the weights are not powers of two, so every product and every partial sum "
                                      "of the reference's chain is rounded: each of the chain's adds runs either "
                                      "as a binary64 add or as its exact fixed-point image"}}

    # ---- the reference's own CUDA stencil (Cxx11/stencil-cuda.cu, sm_103a) beside ours ----
    comparator = None
    if not args.no_comparator and rank == 0:
        comparator = reference_cuda_rate(torch, kg, n, r)

    # ---- batched: the seeded 256-grid configuration in one persistent kernel per launch ----
    batched = None
    if not args.no_batch:
        from kernels_gb300.workloads import batch_specs, shard
        batched = {}
        all_specs = batch_specs()
        for dname, dt in (("fp64", kg.FP64), ("fp32c", kg.FP32C)):
            # independent grids, split by cost: no exchange
            specs = [all_specs[k] for k in shard(all_specs, rank, world, dname)]
            grids = []
            for p, rr, nn in specs:
                a, bb, o = kg.alloc(nn, dt)
                kg.init(a, o)
                grids.append((p, rr, a, bb, o))
            bt = kg.Batch(grids, tuned=True)
            bt.run(args.batch_iterations, graph=True)  # tuning, graph capture and warm-up
            for p, rr, a, bb, o in grids:
                kg.init(a, o)
            tb = max_over_ranks(bt.run(args.batch_iterations, graph=True))
            norms = bt.norms()
            fl_b = sum(kg.flops(p, rr, nn) for p, rr, nn in all_specs) * args.batch_iterations  # whole batch
            batched[dname] = {"value": round(fl_b / tb / 1e9, 3), "unit": "GFLOP/s",
                              "seconds": round(tb, 5), "launches": bt.launches(args.batch_iterations),
                              "norms_ok": all(abs(x - 2.0 * (args.batch_iterations + 1)) <= 1e-8 for x in norms)}
            bt.close()
            # the same grids one after another through the single-grid path (tuned), for comparison
            tseq = 0.0
            for p, rr, a, bb, o in grids:
                kg.init(a, o)
                tseq += kg.run(p, rr, args.batch_iterations, a, bb, o, tuned=True).elapsed_s
            tseq = max_over_ranks(tseq)
            batched[dname]["one_grid_at_a_time"] = {"value": round(fl_b / tseq / 1e9, 3), "seconds": round(tseq, 5)}
            del grids
            torch.cuda.empty_cache()
        batched["workload"] = (f"{len(all_specs)} grids, n log-uniform in [128, 4096], R uniform in 1..4, star/grid 50/50 "
                               f"(seed {20260101}), {args.batch_iterations} timed iterations, tuned depth per grid, "
                               f"one CUDA graph; split across {world} rank(s) by cost, timed by the slowest")
        batched["scaling"] = "strong"

    # ---- end to end through the host-buffer C-ABI call (copies inside the timed region) ----
    e2e = None
    if not args.no_e2e:
        e2e_iters = args.e2e_iterations
        h_in = torch.empty((n, n), dtype=torch.float64).pin_memory()
        h_out = torch.zeros((n, n), dtype=torch.float64).pin_memory()
        h_in.copy_(torch.arange(n, dtype=torch.float64)[:, None] + torch.arange(n, dtype=torch.float64)[None, :])
        # Warm-up call (allocator, module load), then the timed calls back to back: the host link
        # drops to a slower state after about half a second without traffic, and a pause between
        # calls (re-zeroing out on the host) would time its wake-up. out accumulates instead: every
        # call adds 2(K+1) to each interior point, so its norm is known.
        kg.run_host(pattern, r, 1, h_in, h_out)
        te, ev, norm_ok, each = 0.0, 0.0, True, []
        for step in range(args.e2e_steps):
            barrier()
            t0 = time.perf_counter()
            res = kg.run_host(pattern, r, e2e_iters, h_in, h_out)
            each.append(max_over_ranks(time.perf_counter() - t0))
            te += each[-1]
            ev += res["kernel_s"]
            norm_ok &= abs(res["norm"] - (4.0 + 2.0 * (e2e_iters + 1) * (step + 1))) <= 1e-8
        steps_e = args.e2e_steps
        # The median call: the host link of a shared machine stalls now and then (one call in a few
        # can take several times as long); every call's time and the mean are listed beside it.
        t_med = sorted(each)[len(each) // 2]
        e2e = {"value": round(world * fl * (e2e_iters + 1) / t_med / 1e9, 3), "unit": "GFLOP/s",
               "statistic": "median of the timed calls",
               "mean_value": round(world * fl * (e2e_iters + 1) * steps_e / te / 1e9, 3),
               "h2d_bytes_per_step": 2 * n * n * 8, "d2h_bytes_per_step": n * n * 8 + 8,
               "step": f"one prk_gb300_run_host call from pinned host buffers: in and out copied to the "
                       f"device in bands of rows, each band's {e2e_iters + 1} fused applications in one launch "
                       f"and its out copied back, overlapped across bands; device norm",
               "steps": steps_e, "seconds_per_step": round(te / steps_e, 4),
               "seconds_each": [round(x, 4) for x in each],
               "evaluation_seconds_per_step": round(ev / steps_e, 4),
               "norm_ok": bool(norm_ok)}

    clocks.__exit__(None, None, None)
    peak, peak_kind = hbm_peak()
    b64 = algorithmic_bytes(n, r, True)
    b32 = algorithmic_bytes(n, r, False)
    ach64 = b64 * args.steps / t64 / 1e9
    ach32 = b32 * args.steps / t32 / 1e9
    prof = profiled_traffic()
    traffic = prof.get("fp64_star2_n16384_bytes_per_launch")
    traffic_src = ("profiles/traffic.json: " + prof.get("source", "")) if traffic else None
    value = world * fl * args.steps / t64 / 1e9
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * t64 / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"PRK star stencil R={r}, n={n}, FP64, one fused application (out += S(in), "
                               f"in_next = in + 1) per step", "pattern": "star", "radius": r, "n": n,
                   "l2": (f"inputs larger than L2 ({8 * n * n / 1e9:.1f} GB per array), no flush" if 8 * n * n > L2_BYTES
                          else "inputs within L2 (a small case, not the benchmark)"),
                   "parallelism": f"replicas x{world}"},
        "hbm_gbs": round(world * ach64, 2),
        "norm_check": norm_ok,
        "roofline": {"bound": "hbm", "achieved": round(ach64, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(ach64 / peak, 4), "peak_source": peak_kind,
                     "traffic": traffic, "traffic_source": traffic_src, "algorithmic_bytes_per_launch": b64},
        "fp32c": {"value": round(world * fl * args.steps / t32 / 1e9, 3), "unit": "GFLOP/s",
                  "ms_per_step": round(1e3 * t32 / args.steps, 4), "hbm_gbs": round(ach32, 2),
                  "roofline_frac": round(ach32 / peak, 4), "rel_err_vs_fp64": rel32,
                  "rel_err_note": "max over 256 sampled interior points of |hi+lo - fp64| / |fp64|; the FP64 path "
                                  "is bit-identical to the strict-order reference (parity tests)",
                  "norm_check": abs(nrm32 - 2.0 * apps) <= 1e-8, "algorithmic_bytes_per_launch": b32},
        "temporal": {"unit": "GFLOP/s", "what": "the same workload with `depth` applications per launch on a tile "
                                                "held in shared memory (temporal blocking); keys are depths, the "
                                                "largest a whole run of that many applications in one launch",
                     **temporal} if not args.no_temporal else None,
        "grid2": grid2,
        "gpu_comparator": comparator,
        "batched": batched,
        "clocks": clocks.summary(),
        "gpu_launches": args.steps,
    }
    if e2e:
        line["e2e"] = e2e
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_port_rate(pattern, r, n, args.cpu_applications)
        line["cpu_baseline"] = {"value": round(cb["gflops"], 3), "unit": "GFLOP/s", "cores": cb["threads"],
                                "kind": "port",
                                "sample": f"{args.cpu_applications} applications of star R=2 at n={n} "
                                          f"({cb['seconds']:.2f} s), stencil-openmp loop restated in C with "
                                          f"-O3 -ffast-math -fopenmp"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--radius", type=int, default=R_DEFAULT)
    ap.add_argument("--e2e-iterations", type=int, default=100)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-applications", type=int, default=100)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-temporal", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-grid", action="store_true")
    ap.add_argument("--no-comparator", action="store_true")
    ap.add_argument("--batch-iterations", type=int, default=50)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)  # at least 3 untimed warm-up steps
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
