"""One grid split across ranks in row slabs (kernels_gb300.decomp), on CPU gloo ranks.

Each rank runs the oracle on its slab (oracle prk_oracle_apply_rows, the generator's strict order)
and exchanges R-row halos with its neighbours through torch.distributed point-to-point messages, as
MPI1/Stencil/stencil.c:338-420 does with MPI. The owned rows gathered from the ranks must equal the
single-grid oracle run bit for bit on the reference's CI cases (ci/build-run-prk.sh: 10 iterations,
n=200, star and grid R=1..5) and on n=1000 star R=2, with two and three ranks, at depth 1 (an
exchange before every application, as the reference) and depth 4 (one exchange per four
applications: in evolves pointwise, so the R-row halo serves them all). The norm is each rank's sum
of |out|, summed across ranks (MPI1/Stencil/stencil.c:425-436), and must pass the reference's check.
"""
import math
import os
import socket

import numpy as np
import pytest

from kernels_gb300 import FP64, PrkError
from kernels_gb300.decomp import Slab, slab_rows

CASES = [(p, r, 200, 10) for p in (0, 1) for r in range(1, 6)] + [(0, 2, 1000, 10)]


def test_slab_rows_follow_the_reference_leftover_rule():
    # MPI1/Stencil/stencil.c:232-241: the first n % P ranks take one row more
    assert [slab_rows(10, k, 3) for k in range(3)] == [(0, 4), (4, 7), (7, 10)]
    assert [slab_rows(9, k, 3) for k in range(3)] == [(0, 3), (3, 6), (6, 9)]
    for n, world in ((200, 3), (1000, 7), (16384, 8), (5, 5)):
        spans = [slab_rows(n, k, world) for k in range(world)]
        assert spans[0][0] == 0 and spans[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
        sizes = [e - b for b, e in spans]
        assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)


def test_slab_halo_geometry():
    s = Slab.of(200, 3, 1, 3)
    assert (s.row_begin, s.row_end, s.halo_begin, s.halo_end) == (67, 134, 64, 137)
    assert s.own == slice(3, 70)
    assert s.up() == (0, slice(3, 6), slice(0, 3))
    assert s.down() == (2, slice(67, 70), slice(70, 73))
    first, last = Slab.of(200, 3, 0, 3), Slab.of(200, 3, 2, 3)
    assert first.up()[0] is None and first.halo_begin == 0
    assert last.down()[0] is None and last.halo_end == 200


def test_slab_rejects_what_the_reference_rejects():
    with pytest.raises(PrkError):
        Slab.of(12, 5, 0, 3)  # 4 rows per rank, fewer than R = 5
    with pytest.raises(PrkError):
        Slab.of(3, 1, 3, 4)  # no rows for the last rank
    with pytest.raises(PrkError):
        Slab.of(9, 5, 0, 1)  # 2R+1 > n
    with pytest.raises(ValueError):
        slab_rows(10, 3, 3)


class OracleBackend:
    """The slabs' stencil work on the CPU oracle (test infrastructure)."""

    def __init__(self):
        import torch
        from oracle import prk_oracle as po
        self.torch, self.po = torch, po

    def alloc(self, slab, dtype):
        assert dtype == FP64
        t = self.torch
        return (t.zeros((slab.rows, slab.n), dtype=t.float64), t.zeros((slab.rows, slab.n), dtype=t.float64),
                t.zeros((slab.rows, slab.n), dtype=t.float64))

    def apply(self, pattern, slab, apps, cur, nxt, out):
        a = cur.numpy().copy()
        o = out.numpy()
        for _ in range(apps):  # the halo rows advance here as the neighbours advance theirs
            self.po.apply_rows(pattern, slab.radius, slab.n, slab.halo_begin, slab.row_begin, slab.row_end, a, o)
            a += 1.0
        nxt.numpy()[slab.own] = a[slab.own]

    def l1_sum(self, slab, out):
        r, n = slab.radius, slab.n
        lo, hi = max(slab.row_begin, r) - slab.halo_begin, min(slab.row_end, n - r) - slab.halo_begin
        return math.fsum(np.abs(out.numpy()[lo:hi, r:n - r]).ravel().tolist()) if hi > lo else 0.0

    def synchronize(self):
        pass


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, depth, q):
    import torch.distributed as dist
    from kernels_gb300.decomp import SlabRun
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out = []
        for pattern, r, n, k in CASES:
            run = SlabRun(pattern, r, n, FP64, dist=dist, backend=OracleBackend(), depth=depth)
            run.init()
            run.run(k)
            nrm = run.norm()
            s = run.slab
            out.append((s.row_begin, s.row_end, run.out.numpy()[s.own].copy(), run.in_.numpy()[s.own].copy(),
                        nrm, run.launches))
        q.put((rank, out))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,depth", [(2, 1), (3, 1), (3, 4)])
def test_gloo_ranks_match_the_single_grid_oracle(world, depth):
    import torch.multiprocessing as mp
    from oracle import prk_oracle as po
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, depth, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = dict(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for c, (pattern, r, n, k) in enumerate(CASES):
        in_ref, out_ref = po.run(pattern, r, n, k)
        got_out = np.zeros((n, n))
        got_in = np.zeros((n, n))
        for rank in range(world):
            b, e, o, i, nrm, launches = results[rank][c]
            got_out[b:e] = o
            got_in[b:e] = i
            assert launches == 1 + -(-k // depth)  # application 0, then launches of `depth`
        assert np.array_equal(got_out.view(np.uint64), out_ref.view(np.uint64)), (pattern, r, n)
        assert np.array_equal(got_in, in_ref)
        norms = {results[rank][c][4] for rank in range(world)}
        assert len(norms) == 1  # every rank holds the reduced value
        nrm = norms.pop()
        assert abs(nrm - po.norm(r, out_ref)) <= 1e-13 * nrm
        assert abs(nrm - 2.0 * (k + 1)) <= 1e-8
