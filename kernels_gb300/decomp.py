"""One PRK grid split across ranks in row slabs, with a halo exchange between applications.

The reference's distributed stencil (MPI1/Stencil/stencil.c) splits the grid into blocks, one per
rank (:199-268, leftover rows and columns to the first ranks), and before every application each
rank sends its outermost R rows and columns to its neighbours and receives theirs into its halo
(:338-404). It then applies the stencil to the interior points of its block and adds one to its
block of `in` (:406-420); at the end the time is the maximum over ranks and the norm the sum of the
ranks' norms (:425-436).

Here a rank owns whole rows: rank k of P owns the grid rows [row_begin, row_end) given by the
reference's leftover rule along one dimension (slab_rows). A slab's halo is then R contiguous rows
of each neighbour's slab, so every exchange is one contiguous message each way with no packing, and
the slab is one row-major buffer that the tile kernels take as it is (prk_gb300_slab_run). The halo
volume per rank is 2 R n values, against 2 R (n/Px + n/Py) for blocks; with n in the tens of
thousands and a handful of ranks per node that is a few hundred kilobytes per exchange.

`in` evolves pointwise (in += 1 after every application), so a slab launch can carry `depth`
applications on one R-row halo: the kernel advances the halo rows it holds exactly as the
neighbours advance theirs. The exchange then runs once per launch (every application at depth 1,
as the reference does). Every application still reads the current `in` values of every tap.

The exchange uses torch.distributed point-to-point messages (isend/irecv): NCCL with device tensors
on GPUs, gloo with host tensors on CPUs. The ranks' stencil work goes through a backend object:
DeviceBackend runs the slabs on this rank's GPU through the C ABI; the tests give the CPU oracle
instead, with gloo ranks.
"""
from __future__ import annotations

from dataclasses import dataclass

from . import FP32C, FP64, PrkError, slab_norm, slab_run

# message tags, one per direction (the reference uses 99/101 for its y-direction exchange)
TAG_DOWN, TAG_UP = 101, 99


def slab_rows(n: int, rank: int, world: int) -> tuple[int, int]:
    """Grid rows [row_begin, row_end) of rank `rank` of `world`: n // world rows each, one more for
    the first n % world ranks (MPI1/Stencil/stencil.c:232-241, along the rows)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank or world size")
    width, leftover = divmod(n, world)
    if rank < leftover:
        begin = (width + 1) * rank
        return begin, begin + width + 1
    begin = (width + 1) * leftover + width * (rank - leftover)
    return begin, begin + width


@dataclass(frozen=True)
class Slab:
    """Rank `rank`'s share of an n x n grid for a stencil of radius R: it owns grid rows
    [row_begin, row_end) and its buffers hold rows [halo_begin, halo_end)."""
    n: int
    radius: int
    rank: int
    world: int
    row_begin: int
    row_end: int
    halo_begin: int
    halo_end: int

    @staticmethod
    def of(n: int, radius: int, rank: int, world: int) -> "Slab":
        """The slab, with the reference's checks: every rank has work, and at least R rows so that a
        halo comes from the next rank alone (MPI1/Stencil/stencil.c:243-274)."""
        if n < 2 * radius + 1:
            raise PrkError(-1, f"stencil radius {radius} too large for n={n}")
        b, e = slab_rows(n, rank, world)
        if e - b < 1:
            raise PrkError(-1, f"rank {rank} has no work to do (n={n}, {world} ranks)")
        if world > 1 and e - b < radius:
            raise PrkError(-1, f"rank {rank} has {e - b} rows, fewer than the stencil radius {radius}")
        return Slab(n, radius, rank, world, b, e, max(0, b - radius), min(n, e + radius))

    @property
    def rows(self) -> int:
        """Rows the buffers hold (owned rows and halo)."""
        return self.halo_end - self.halo_begin

    @property
    def own(self) -> slice:
        """The owned rows as buffer rows."""
        return slice(self.row_begin - self.halo_begin, self.row_end - self.halo_begin)

    def up(self) -> tuple[int | None, slice, slice]:
        """(neighbour above, the owned rows it needs, the halo rows it fills), buffer rows."""
        if self.rank == 0:
            return None, slice(0, 0), slice(0, 0)
        o = self.row_begin - self.halo_begin
        return self.rank - 1, slice(o, o + self.radius), slice(0, o)

    def down(self) -> tuple[int | None, slice, slice]:
        """(neighbour below, the owned rows it needs, the halo rows it fills), buffer rows."""
        if self.rank == self.world - 1:
            return None, slice(0, 0), slice(0, 0)
        e = self.row_end - self.halo_begin
        return self.rank + 1, slice(e - self.radius, e), slice(e, self.rows)


def exchange(slab: Slab, buf, dist, group=None) -> None:
    """Fill the halo rows of `buf` (a [slab.rows, n] tensor holding the current `in`) from the
    neighbours' owned rows, and send them the rows they need (MPI1/Stencil/stencil.c:338-371, rows
    only). Non-blocking sends and receives, all posted before any wait, so no ordering between the
    ranks can deadlock."""
    reqs = []
    for nbr, send_rows, recv_rows, send_tag, recv_tag in ((*slab.up(), TAG_UP, TAG_DOWN),
                                                          (*slab.down(), TAG_DOWN, TAG_UP)):
        if nbr is None:
            continue
        reqs.append(dist.irecv(buf[recv_rows], src=nbr, group=group, tag=recv_tag))
        reqs.append(dist.isend(buf[send_rows].contiguous(), dst=nbr, group=group, tag=send_tag))
    for r in reqs:
        r.wait()


class DeviceBackend:
    """The slabs' stencil work on this rank's GPU through the C ABI (prk_gb300_slab_run and
    prk_gb300_slab_norm)."""

    def __init__(self, device=None):
        import torch
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)

    def alloc(self, slab: Slab, dtype: int):
        t = self.torch
        fdt = t.float64 if dtype == FP64 else t.float32
        shape_out = (slab.rows, slab.n) if dtype == FP64 else (slab.rows, slab.n, 2)
        return (t.empty((slab.rows, slab.n), dtype=fdt, device=self.device),
                t.empty((slab.rows, slab.n), dtype=fdt, device=self.device),
                t.zeros(shape_out, dtype=fdt, device=self.device))

    def apply(self, pattern: int, slab: Slab, apps: int, cur, nxt, out) -> None:
        slab_run(pattern, slab.radius, slab.n, apps, slab.row_begin, slab.row_end, cur, nxt, out)

    def l1_sum(self, slab: Slab, out) -> float:
        return slab_norm(slab.radius, slab.n, slab.row_begin, slab.row_end, out)

    def synchronize(self) -> None:
        self.torch.cuda.synchronize(self.device)


class SlabRun:
    """A PRK run (Cxx11/stencil-openmp.cc:182-258 semantics: in = i+j, out = 0, iterations+1
    applications each followed by in += 1, the norm over the interior checked against
    2(iterations+1)) on one grid split across the ranks of `group` in row slabs.

    Each rank keeps its slab in two `in` buffers (ping-pong) and one `out` buffer. A launch of
    `depth` applications is preceded by an exchange of the current `in`'s halo rows."""

    def __init__(self, pattern: int, radius: int, n: int, dtype: int = FP64, dist=None, group=None,
                 backend=None, depth: int = 1):
        if depth < 1:
            raise PrkError(-1, "depth must be >= 1")
        if dtype not in (FP64, FP32C):
            raise PrkError(-1, f"dtype {dtype} is not FP64 or FP32C")
        self.dist, self.group = dist, group
        rank = dist.get_rank(group) if dist else 0
        world = dist.get_world_size(group) if dist else 1
        self.pattern, self.dtype, self.depth = pattern, dtype, depth
        self.slab = Slab.of(n, radius, rank, world)
        self.backend = backend if backend is not None else DeviceBackend()
        self.bufs = list(self.backend.alloc(self.slab, dtype))
        self.cur = 0
        self.launches = 0

    @property
    def out(self):
        return self.bufs[2]

    @property
    def in_(self):
        """The buffer holding the current `in`."""
        return self.bufs[self.cur]

    def init(self) -> None:
        """in(i,j) = i+j on the owned rows, out = 0 (MPI1/Stencil/stencil.c:302-305 initialises
        each rank's own block); the halo rows come from the neighbours at the first exchange."""
        s = self.slab
        t = self.bufs[0]
        rows = t.new_tensor(range(s.row_begin, s.row_end)).reshape(-1, 1)
        cols = t.new_tensor(range(s.n)).reshape(1, -1)
        t.zero_()
        t[s.own] = rows + cols
        self.bufs[2].zero_()
        self.cur = 0

    def _launch(self, apps: int) -> None:
        if self.slab.world > 1:
            self.backend.synchronize()  # the previous launch has written the rows to send
            exchange(self.slab, self.bufs[self.cur], self.dist, self.group)
        self.backend.apply(self.pattern, self.slab, apps, self.bufs[self.cur], self.bufs[self.cur ^ 1], self.out)
        self.cur ^= 1
        self.launches += 1

    def run(self, iterations: int) -> float:
        """Application 0 (untimed, as the reference's warm-up iteration), then `iterations` timed
        applications in launches of `depth` (the remainder in a shorter one). Returns the slowest
        rank's seconds for the timed applications."""
        import time
        if iterations < 1:
            raise PrkError(-1, "iterations must be >= 1")
        self._launch(1)
        self._barrier()
        t0 = time.perf_counter()
        left = iterations
        while left > 0:
            a = min(self.depth, left)
            self._launch(a)
            left -= a
        self._barrier()
        return self._max(time.perf_counter() - t0)

    def norm(self) -> float:
        """The L1 norm over the whole grid's interior / (n-2R)^2: each rank's sum, then their sum
        (MPI1/Stencil/stencil.c:425-436)."""
        s = self.slab
        local = self.backend.l1_sum(s, self.out)
        total = self._sum(local)
        return total / float((s.n - 2 * s.radius) ** 2)

    def _barrier(self) -> None:
        self.backend.synchronize()
        if self.dist and self.slab.world > 1:
            self.dist.barrier(group=self.group)

    def _reduce(self, x: float, op) -> float:
        if not self.dist or self.slab.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device=self.out.device)
        self.dist.all_reduce(t, op=op, group=self.group)
        return float(t.item())

    def _max(self, x: float) -> float:
        return self._reduce(x, self.dist.ReduceOp.MAX) if self.dist else x

    def _sum(self, x: float) -> float:
        return self._reduce(x, self.dist.ReduceOp.SUM) if self.dist else x
