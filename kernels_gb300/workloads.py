"""Seeded synthetic workloads for the stencil configurations (no external dataset exists for PRK), and
the split of a batch across ranks (its grids are independent, so ranks share no data), weighed by
each grid's cost.

batch_specs(): the batched configuration: 256 independent grids with n log-uniform in [128, 4096],
radius uniform in {1, 2, 3, 4}, star or grid 50/50, from a fixed seed. Every grid starts from the
PRK initial field (in = i+j, out = 0), so every norm must come out as 2*(iterations+1).
"""
from __future__ import annotations

import math

import numpy as np

BATCH_SEED = 20260101


# Measured time per point and application of each stencil on one GB300, as PRK GFLOP/s of tuned
# runs at n = 32768 (kernels_gb300.configs sweep): the cost model of the split below. The FP64
# stencils with power-of-two weights take the exact integer routes and run an order of magnitude
# faster than the ones whose every add is rounded; FP32C is fast for all of them.
SWEEP_GFLOPS = {
    "fp64": {(0, 1): 18116, (0, 2): 27871, (0, 3): 1930, (0, 4): 2061, (0, 5): 2027,
             (1, 1): 28738, (1, 2): 2439, (1, 3): 2394, (1, 4): 2237, (1, 5): 2175},
    "fp32c": {(0, 1): 13915, (0, 2): 16571, (0, 3): 17538, (0, 4): 17514, (0, 5): 17170,
              (1, 1): 17556, (1, 2): 22891, (1, 3): 27141, (1, 4): 33038, (1, 5): 33318},
}


def grid_cost(pattern: int, radius: int, n: int, dtype: str = "fp64") -> float:
    """Seconds per application of one grid under the cost model: its interior points times PRK's flop
    count per point ((2 stencil_size + 1), Cxx11/stencil-openmp.cc:253-255) over the stencil's
    measured rate."""
    size = 4 * radius + 1 if pattern == 0 else (2 * radius + 1) ** 2
    return (n - 2 * radius) ** 2 * (2 * size + 1) / (SWEEP_GFLOPS[dtype][(pattern, radius)] * 1e9)


def shard(items: list, rank: int, world: int, dtype: str = "fp64", costs: list | None = None) -> list[int]:
    """Indices of the items (pattern, radius, n) rank `rank` of `world` owns: a greedy split by cost
    (largest first, each to the least-loaded rank), so that ranks finish together. The cost of a grid
    is `costs[k]` when given (e.g. the autotuner's measured seconds), else grid_cost for `dtype`.
    Every index goes to exactly one rank and every rank computes the same split without talking to
    the others."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank or world size")
    cost = costs if costs is not None else [grid_cost(p, r, n, dtype) for p, r, n in items]
    order = sorted(range(len(items)), key=lambda k: (-cost[k], k))
    load = [0.0] * world
    owner = [0] * len(items)
    for k in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[k] = r
        load[r] += cost[k]
    return [k for k in range(len(items)) if owner[k] == rank]


def batch_specs(count: int = 256, seed: int = BATCH_SEED, n_lo: int = 128, n_hi: int = 4096,
                radii=(1, 2, 3, 4)) -> list[tuple[int, int, int]]:
    """(pattern, radius, n) per grid; pattern 0 = star, 1 = grid."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        r = int(rng.choice(radii))
        p = int(rng.integers(0, 2))
        specs.append((p, r, max(n, 2 * r + 1)))
    return specs
