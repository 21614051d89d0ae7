"""Sharding of one MC iteration over ranks (one process per GPU).

The reference parallelises iterateMC with MPI (source/iteration_mod.f90:729-753,
:953): each rank transports its share of the packets of every source, then one
MPI_Allreduce sums Jste (and the escape tallies) so that every rank sees the
whole radiation field; the per-cell phases are independent per cell.  Here the
packets of an iteration are numbered globally (packet k draws from Philox stream
(seed, counter_base + k)), so a rank's share is a contiguous counter range and
the sum over ranks of their estimators equals the single-rank run packet for
packet; the only exchange is the sum of J.

``shard_packets`` gives a rank its range; ``allreduce_sum`` sums an estimator
array over the process group (NCCL on device tensors, gloo on host tensors);
``transport_sharded`` is one rank's transport phase of a sharded iteration
through libmcx: its share of the packets, then the sum of Jste and of the
escape tallies over the group, written back into the rank's context (every
rank then balances every cell, as each MPI rank of the reference holds the
whole grid).
"""
from __future__ import annotations

import numpy as np


def shard_packets(n_total: int, rank: int, world: int) -> tuple[int, int]:
    """(first packet id, packet count) of `rank` among `world` ranks: contiguous, sizes differing by at most 1."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"shard_packets: rank {rank} outside a world of {world}")
    base, extra = divmod(int(n_total), world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def allreduce_sum(a, group=None):
    """Sum a numpy array or torch tensor over the ranks of the default (or given) process group, in place
    where the input is a tensor; returns the summed array."""
    import torch
    import torch.distributed as dist
    if isinstance(a, np.ndarray):
        t = torch.from_numpy(np.ascontiguousarray(a))
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        return t.numpy()
    dist.all_reduce(a, op=dist.ReduceOp.SUM, group=group)
    return a


def transport_sharded(ctx, n_total: int, seed: int, counter_base: int, precision: int, group=None, istar: int = 1,
                      zero: bool = True, reduce: bool = True, **opts):
    """The transport phase of one iteration sharded over the ranks of `group`
    (source/iteration_mod.f90:729-753 and the MPI_Allreduce of Jste and
    escapedPackets at :953): this rank transports packets
    [counter_base + first, + count) of source `istar`'s n_total (deltaE =
    Lstar(istar) / n_total on every rank), then (with `reduce`) Jste and the
    escape tallies are summed over the group and put back into the context; the
    returned statistics are the group's totals.  Several sources: `zero` for
    the first only and `reduce` after the last, so that each rank's estimators
    hold its share of every source before the one sum."""
    import torch
    import torch.distributed as dist
    from . import abi
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    first, count = shard_packets(n_total, rank, world)
    st = ctx.transport(count, seed=seed, counter_base=counter_base + first, precision=precision, zero=zero,
                       n_photons_norm=n_total, istar=istar, **opts)
    for arr in ((abi.ARR_JSTE, abi.ARR_ESCAPED) if reduce else ()):
        ctx.put(arr, allreduce_sum(ctx.get(arr), group))
    names = ("crossings", "interactions", "absorptions", "scatterings", "escaped", "line_escapes", "trapped",
             "emissions")
    t = torch.tensor([getattr(st, k) for k in names], dtype=torch.int64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    for k, v in zip(names, t.tolist()):
        setattr(st, k, v)
    q = torch.tensor([st.q_phot], dtype=torch.float64)
    dist.all_reduce(q, op=dist.ReduceOp.SUM, group=group)
    st.q_phot = float(q.item())
    return st
