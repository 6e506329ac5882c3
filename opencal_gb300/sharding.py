"""Multi-GPU sharding of the cellular-automaton step: one process per GPU,
torch.distributed for the exchanges, and no collective on any data path
that does not need one.

The path shards two ways:

* **Instances** (calibration ensembles, scenario batches).  The automata are
  independent; each rank takes a contiguous share of the instances, balanced
  by cell count (``shard_instances``), and runs its share alone.  The only
  exchange is the gather of per-instance results -- losses and gradients, a
  few scalars each -- in global instance order (``gather_instances``,
  ``ShardedEnsemble``).

* **One grid by row slabs** (``RowSlabs``, ``halo_exchange``,
  ``run_row_slabs``).  Rank r owns rows [lo_r, hi_r) and keeps
  ``halo = k * radius`` extra rows on every side that borders another rank
  (radius: how many rows a cell's new state reaches per step).  Every k
  steps the ranks swap those rows with their neighbours (point-to-point
  send/receive of contiguous row blocks), then run k steps on their
  extended slab alone.  A slab's artificial edge spoils `radius` rows per
  step, so after k steps the damage has crossed the halo and stops short of
  the owned rows, which stay exact.  At the grid's own top and bottom edges
  a slab keeps no halo and uses the grid's flat boundary.  Concatenating
  the owned rows in rank order gives the grid in its row-major order (an
  active-cell list concatenates the same way, each rank's rows shifted by
  lo_r).  Grids whose rows wrap (toroidal) are not sliced this way.

Nothing here uses NVLink or TMA multicast: the exchanges are
torch.distributed point-to-point and all-gather calls (NCCL between GPUs,
gloo on the CPU, where the tests run them).
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np


# ---------------------------------------------------------------- instances

def shard_instances(cells: Sequence[int], world: int) -> list[tuple[int, int]]:
    """Contiguous [start, end) ranges of instances for each of `world`
    ranks, balanced by cell count: rank r's range ends at the first instance
    boundary where the running total reaches (r + 1) / world of all cells.
    Every rank gets at least one instance while there are enough."""
    n = len(cells)
    if world <= 0:
        raise ValueError("world must be positive")
    csum = np.cumsum(np.asarray(cells, dtype=np.float64))
    total = float(csum[-1]) if n else 0.0
    bounds = [0]
    for r in range(1, world):
        cut = int(np.searchsorted(csum, total * r / world, side="left")) + 1 if n else 0
        if n >= world:
            cut = min(max(cut, bounds[-1] + 1), n - (world - r))
        else:
            cut = min(max(cut, bounds[-1]), n)
        bounds.append(cut)
    bounds.append(n)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def gather_instances(local: np.ndarray, ranges: Sequence[tuple[int, int]], dist, device="cpu") -> np.ndarray:
    """All-gather of per-instance rows: `local` holds this rank's rows
    (shape (end - start, ...)); returns every instance's rows in global
    order on every rank.  Rows are padded to the largest share for the
    collective and trimmed afterwards."""
    import torch
    local = np.ascontiguousarray(local)
    if dist is None:
        return local.copy()
    world = dist.get_world_size()
    width = max(e - s for s, e in ranges)
    tail = local.shape[1:]
    buf = torch.zeros((width,) + tail, dtype=torch.float64, device=device)
    if len(local):
        buf[: len(local)] = torch.from_numpy(local.astype(np.float64)).to(device)
    parts = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf)
    out = [parts[r][: ranges[r][1] - ranges[r][0]].cpu().numpy() for r in range(world)]
    return np.concatenate(out, axis=0).astype(local.dtype if local.size else np.float64)


def sharded_map(fn: Callable[[int], np.ndarray], cells: Sequence[int], dist, device="cpu") -> np.ndarray:
    """fn(i) -> 1-D array of results of instance i, evaluated for this rank's
    share of the instances and gathered in instance order on every rank."""
    rank = dist.get_rank() if dist is not None else 0
    world = dist.get_world_size() if dist is not None else 1
    ranges = shard_instances(cells, world)
    s, e = ranges[rank]
    rows = [np.atleast_1d(np.asarray(fn(i), dtype=np.float64)) for i in range(s, e)]
    width = max((len(r) for r in rows), default=0)
    if dist is not None:
        import torch
        w = torch.tensor([width], dtype=torch.float64, device=device)
        dist.all_reduce(w, op=dist.ReduceOp.MAX)
        width = int(w.item())
    local = np.zeros((e - s, width))
    for k, r in enumerate(rows):
        local[k, : len(r)] = r
    return gather_instances(local, ranges, dist, device=device)


class ShardedEnsemble:
    """A SCIDDICA-T calibration ensemble split by instance across ranks:
    each rank holds an ``opencal_gb300.ensemble.Ensemble`` of its share on
    its own GPU; ``loss_grad`` runs the batched forward + adjoint there and
    all-gathers the losses and (dL/dp_r, dL/dp_eps) of every instance."""

    def __init__(self, dims, params, zs, hs, steps: int, dist, device="cuda"):
        from .ensemble import Ensemble
        self.dist = dist
        self.rank = dist.get_rank() if dist is not None else 0
        world = dist.get_world_size() if dist is not None else 1
        self.ranges = shard_instances([r * c for r, c in dims], world)
        s, e = self.ranges[self.rank]
        self.start, self.end = s, e
        self.device = device
        self.local = Ensemble(dims[s:e], np.asarray(params)[s:e], zs[s:e], hs[s:e], steps, device=device)

    def set_params(self, params):
        self.local.set_params(np.asarray(params)[self.start:self.end])

    def local_target(self, targets):
        """This rank's share of per-instance target maps, packed for its ensemble."""
        return self.local.pack(targets[self.start:self.end])

    def loss_grad(self, local_target):
        loss, grad = self.local.loss_grad(local_target)[:2]
        rows = np.concatenate([np.asarray(loss).reshape(-1, 1), np.asarray(grad).reshape(-1, 2)], axis=1)
        full = gather_instances(rows, self.ranges, self.dist, device=self.device)
        return full[:, 0], full[:, 1:3]

    def close(self):
        self.local.close()


# ---------------------------------------------------------------- row slabs

class RowSlabs:
    """Row partition of a rows-high grid over `world` ranks with halos of
    k * radius rows towards neighbouring ranks."""

    def __init__(self, rows: int, world: int, k: int, radius: int):
        if k < 1 or radius < 1:
            raise ValueError("k and radius must be positive")
        self.rows, self.world, self.k, self.radius = rows, world, k, radius
        self.halo = k * radius
        cuts = [rows * r // world for r in range(world + 1)]
        self.owned = [(cuts[r], cuts[r + 1]) for r in range(world)]
        for r, (lo, hi) in enumerate(self.owned):
            if world > 1 and hi - lo < self.halo:
                raise ValueError(f"rank {r} owns {hi - lo} rows, fewer than the halo ({self.halo})")

    def extended(self, r: int) -> tuple[int, int]:
        """Rows [ext_lo, ext_hi) rank r keeps: its own plus the halos."""
        lo, hi = self.owned[r]
        return (lo - self.halo if r > 0 else lo), (hi + self.halo if r < self.world - 1 else hi)

    def owned_slice(self, r: int) -> slice:
        """The owned rows within rank r's extended slab."""
        lo, hi = self.owned[r]
        ext_lo, _ = self.extended(r)
        return slice(lo - ext_lo, hi - ext_lo)


def halo_exchange(ext, slabs: RowSlabs, rank: int, dist) -> None:
    """Refresh rank `rank`'s halo rows of `ext` (a torch tensor holding its
    extended slab, rows first) from its neighbours' owned rows, in place:
    the top halo receives the last `halo` owned rows of rank - 1, the bottom
    halo the first `halo` owned rows of rank + 1; each rank sends the
    matching blocks.  Point-to-point, one message each way per neighbour."""
    if dist is None or slabs.world == 1:
        return
    h = slabs.halo
    own = slabs.owned_slice(rank)
    reqs = []
    recv_top = recv_bot = None
    if rank > 0:
        reqs.append(dist.isend(ext[own.start:own.start + h].contiguous(), dst=rank - 1))
        recv_top = ext[:h].clone()
        reqs.append(dist.irecv(recv_top, src=rank - 1))
    if rank < slabs.world - 1:
        reqs.append(dist.isend(ext[own.stop - h:own.stop].contiguous(), dst=rank + 1))
        recv_bot = ext[own.stop:own.stop + h].clone()
        reqs.append(dist.irecv(recv_bot, src=rank + 1))
    for q in reqs:
        q.wait()
    if recv_top is not None:
        ext[:h] = recv_top
    if recv_bot is not None:
        ext[own.stop:own.stop + h] = recv_bot


def run_row_slabs(step: Callable, grid0: np.ndarray, steps: int, slabs: RowSlabs, dist, device="cpu") -> np.ndarray:
    """Run `steps` steps of a flat-boundary automaton on row slabs:
    step(ext_array, n) -> ext_array after n steps of the rank's extended slab
    (numpy in, numpy out; the slab is an ordinary flat grid of its own).
    Every k steps the halos are exchanged.  Returns the whole grid after the
    run on every rank (owned rows gathered in rank order)."""
    import torch
    rank = dist.get_rank() if dist is not None else 0
    ext_lo, ext_hi = slabs.extended(rank)
    ext = torch.from_numpy(np.ascontiguousarray(grid0[ext_lo:ext_hi])).to(device)
    done = 0
    while done < steps:
        if done:
            halo_exchange(ext, slabs, rank, dist)
        n = min(slabs.k, steps - done)
        ext = torch.from_numpy(np.ascontiguousarray(step(ext.cpu().numpy(), n))).to(device)
        done += n
    mine = ext[slabs.owned_slice(rank)].contiguous()
    if dist is None or slabs.world == 1:
        return mine.cpu().numpy()
    width = max(hi - lo for lo, hi in slabs.owned)
    buf = torch.zeros((width,) + tuple(mine.shape[1:]), dtype=mine.dtype, device=device)
    buf[: mine.shape[0]] = mine
    parts = [torch.empty_like(buf) for _ in range(slabs.world)]
    dist.all_gather(parts, buf)
    return np.concatenate([parts[r][: hi - lo].cpu().numpy() for r, (lo, hi) in enumerate(slabs.owned)], axis=0)
