"""The N>1 path on CPU: two gloo ranks split the seeded batch (independent grids, no exchange) and
agree on the split and on the slowest-rank time, as bench.py does under torchrun."""
import os
import socket

import pytest

from kernels_gb300.workloads import batch_specs, grid_cost, shard


def test_shard_covers_every_grid_once():
    specs = batch_specs()
    for world in (1, 2, 3, 8):
        owned = [shard(specs, r, world) for r in range(world)]
        flat = sorted(k for o in owned for k in o)
        assert flat == list(range(len(specs)))
    with pytest.raises(ValueError):
        shard(specs, 2, 2)


@pytest.mark.parametrize("dtype", ["fp64", "fp32c"])
def test_shard_balances_the_seeded_batch_by_cost(dtype):
    """The split weighs each grid by its cost model (points x flops per point / the stencil's
    measured rate): on the seeded 256-grid batch the most loaded of 2..8 ranks carries within 5% of
    the mean. Weighing by n^2 alone would leave FP64 ranks far apart, a strict grid R=4 point costing
    about 25x a star R=2 point."""
    specs = batch_specs()
    costs = [grid_cost(p, r, n, dtype) for p, r, n in specs]
    for world in range(2, 9):
        loads = [sum(costs[k] for k in shard(specs, r, world, dtype)) for r in range(world)]
        mean = sum(costs) / world
        assert max(loads) <= 1.05 * mean, (world, max(loads) / mean)
    if dtype == "fp64":
        by_n2 = [0.0, 0.0]  # the old weighting by n^2, for contrast
        order = sorted(range(len(specs)), key=lambda k: -specs[k][2] ** 2)
        pts = [0, 0]
        for k in order:
            q = 0 if pts[0] <= pts[1] else 1
            pts[q] += specs[k][2] ** 2
            by_n2[q] += costs[k]
        assert max(by_n2) / (sum(costs) / 2) > 1.05


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    specs = batch_specs()
    mine = shard(specs, rank, world)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    t = torch.tensor([0.5 + rank], dtype=torch.float64)  # each rank's time
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    q.put((rank, gathered, float(t.item())))
    dist.destroy_process_group()


def test_two_gloo_ranks_split_the_batch():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    n = len(batch_specs())
    for rank, gathered, tmax in results:
        assert sorted(gathered[0] + gathered[1]) == list(range(n))
        assert not set(gathered[0]) & set(gathered[1])
        assert tmax == 1.5  # the slowest rank's time, as the benchmark reports
