"""Seeded synthetic workloads for the stencil configurations (no external dataset exists for PRK), and
the split of a batch across ranks (its grids are independent, so ranks share no data).

batch_specs(): the batched configuration: 256 independent grids with n log-uniform in [128, 4096],
radius uniform in {1, 2, 3, 4}, star or grid 50/50, from a fixed seed. Every grid starts from the
PRK initial field (in = i+j, out = 0), so every norm must come out as 2*(iterations+1).
"""
from __future__ import annotations

import math

import numpy as np

BATCH_SEED = 20260101


def shard(items: list, rank: int, world: int) -> list[int]:
    """Indices of the items rank `rank` of `world` owns: a greedy split by work (n^2 per grid, largest
    first, each to the least-loaded rank), so that ranks finish together. Every index goes to exactly
    one rank and every rank computes the same split without talking to the others."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank or world size")
    order = sorted(range(len(items)), key=lambda k: (-items[k][2] ** 2, k))
    load = [0] * world
    owner = [0] * len(items)
    for k in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[k] = r
        load[r] += items[k][2] ** 2
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
