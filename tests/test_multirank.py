"""The N>1 path on CPU: two gloo ranks split the seeded batch (independent grids, no exchange) and
agree on the split and on the slowest-rank time, as bench.py does under torchrun."""
import os
import socket

import pytest

from kernels_gb300.workloads import batch_specs, shard


def test_shard_covers_every_grid_once():
    specs = batch_specs()
    for world in (1, 2, 3, 8):
        owned = [shard(specs, r, world) for r in range(world)]
        flat = sorted(k for o in owned for k in o)
        assert flat == list(range(len(specs)))
        loads = [sum(specs[k][2] ** 2 for k in o) for o in owned]
        assert max(loads) <= 1.05 * min(loads) + max(s[2] ** 2 for s in specs)  # greedy balance
    with pytest.raises(ValueError):
        shard(specs, 2, 2)


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
