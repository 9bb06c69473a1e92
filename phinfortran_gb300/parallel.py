"""Replica parallelism over (omega, q) points: one process per GPU.

Every point is independent, so ranks split the point list and never talk
during the solve; the results are then reduced the way the reference does
it (negf/phinfortran.f90:1500-1519): every rank fills its own entries of a
zero array and an all-reduce SUM over disjoint supports assembles the whole
table on every rank.

``shard_points`` balances contiguous chunks by an estimated cost per point
(n^3 (L + I) for the transport solve); ``shard_indices`` is the default of
the replica runner: without a cost estimate it deals the points out
strided (point i to rank i mod world), because the decimation count I
varies smoothly with the energy (more iterations near subband edges and
band bottoms), so contiguous chunks of an energy grid would give some
ranks the expensive stretches; ``gather_sum`` is the reduction;
``transport_tdb_replicas`` runs `transport_tdb` on this rank's shard and
gathers T_L (and the status words) on every rank.
"""
from __future__ import annotations

import numpy as np


def shard_points(npts, world, rank, cost=None):
    """Indices [lo, hi) of this rank's contiguous shard, balanced by the
    cumulative cost (uniform when cost is None)."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("bad world / rank")
    if npts == 0:
        return 0, 0
    c = np.ones(npts) if cost is None else np.asarray(cost, dtype=np.float64)
    cum = np.concatenate([[0.0], np.cumsum(c)])
    total = cum[-1]
    cuts = [int(np.searchsorted(cum, total * r / world, side="left")) for r in range(world + 1)]
    cuts[0], cuts[-1] = 0, npts
    for r in range(1, world + 1):          # monotone, non-empty where possible
        cuts[r] = max(cuts[r], cuts[r - 1])
    return cuts[rank], cuts[rank + 1]


def shard_indices(npts, world, rank, cost=None):
    """This rank's point indices: strided (rank, rank + world, ...) without a
    cost estimate, else the contiguous cost-balanced chunk of shard_points."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("bad world / rank")
    if cost is None:
        return np.arange(rank, npts, world)
    lo, hi = shard_points(npts, world, rank, cost)
    return np.arange(lo, hi)


def gather_sum(local, lo, hi, npts, group=None, dtype=None, idx=None):
    """Full (npts, ...) array on every rank from each rank's [lo, hi) slice,
    or its entries at the indices idx (all-reduce SUM over disjoint
    supports)."""
    import torch
    import torch.distributed as dist
    local = np.asarray(local)
    full = np.zeros((npts,) + local.shape[1:], dtype=dtype or local.dtype)
    if idx is None:
        full[lo:hi] = local
    else:
        full[np.asarray(idx)] = local
    t = torch.from_numpy(full)
    backend = dist.get_backend(group) if dist.is_initialized() else None
    if backend == "nccl":
        t = t.cuda()
    if dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def transport_tdb_replicas(E, blocks, *, solve=None, group=None, cost=None, **kw):
    """T_L for all points, each rank solving its shard.  ``solve`` defaults
    to phinfortran_gb300.transport_tdb (keyword arguments pass through)."""
    import torch.distributed as dist
    if solve is None:
        from .transport import transport_tdb as solve
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    E = np.asarray(E, dtype=np.float64)
    npts = E.size
    idx = shard_indices(npts, world, rank, cost)
    sub = dict(kw)
    for key in ("qidx", "zero_flag"):
        if sub.get(key) is not None:
            sub[key] = np.asarray(sub[key])[idx]
    if idx.size:
        r = solve(E[idx], blocks, **sub)
        tl, st = r["transl"], r["status"]
    else:
        tl, st = np.zeros(0), np.zeros(0, np.int32)
    return dict(transl=gather_sum(tl, 0, 0, npts, group, np.float64, idx=idx),
                status=gather_sum(st, 0, 0, npts, group, np.int32, idx=idx), shard=idx)
