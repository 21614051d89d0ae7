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
array over the process group (NCCL on device tensors, gloo on host tensors).
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
