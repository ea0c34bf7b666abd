"""Sample sharding across ranks (one GPU per rank, torch.distributed).

Trace-sampling samples are independent, so N ranks each propagate a
contiguous shard of the sample vectors; the only exchange is one all_reduce
of the four T-length population sums. The reference has no distributed layer
(its only parallelism is OpenMP over samples, src/qm_dynamics.f90:322-371);
this keeps its sample average (res%update then res%scale(1/N_samples),
:373-378) while splitting the samples.
"""
from __future__ import annotations

from typing import Callable

import numpy as np

from .observables import Observables


def shard(M: int, rank: int, world: int) -> slice:
    """Contiguous, balanced slice of M samples owned by `rank`."""
    base, extra = divmod(M, world)
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def trace_sampling_sharded(propagate: Callable[[np.ndarray], Observables], zkets: np.ndarray,
                           group=None) -> Observables:
    """Propagate this rank's shard of `zkets` (M x Z) with `propagate` (which
    returns the shard's sample average) and combine across the process group.
    Every rank returns the average over all M samples."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    M = zkets.shape[0]
    sl = shard(M, rank, world)
    n_local = sl.stop - sl.start
    local = propagate(zkets[sl]) if n_local > 0 else None
    if local is not None:
        sums = np.stack([local.P_S, local.P_T0, local.P_Tp, local.P_Tm]) * n_local
    else:
        T = propagate(zkets[:1]).P_S.shape[0]  # shape only
        sums = np.zeros((4, T))
    t = torch.from_numpy(np.ascontiguousarray(sums))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    tot = t.numpy() * (1.0 / M)
    return Observables(tot[0].copy(), tot[1].copy(), tot[2].copy(), tot[3].copy())
