"""I-V sweeps across ranks.

An I-V sweep is a set of independent instances (bias points and parameter
draws), so the multi-GPU path shards instances across ranks -- one process
per GPU, contiguous slices, no data-path collective -- and gathers only the
per-instance results (interface current, steps to steady state) on the host
at the end.  ``torch.distributed`` is used for that gather and for the
bench's barrier/max-time; it works with gloo (CPU tests) and NCCL.
"""
from __future__ import annotations

from typing import Callable, Sequence


def shard(n_total: int, world: int, rank: int) -> range:
    """Contiguous, balanced slice of ``range(n_total)`` owned by ``rank``."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad world/rank")
    base, extra = divmod(n_total, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return range(lo, hi)


def distributed_sweep(params: Sequence, compute: Callable[[list], list], group=None) -> list:
    """Run ``compute`` on this rank's slice of ``params`` and gather the
    per-instance results, in global order, on every rank.

    ``compute(list_of_params) -> list_of_results`` (one result per instance;
    results must be picklable).  Without an initialised process group the
    whole list is computed locally.
    """
    try:
        import torch.distributed as dist
        ready = dist.is_available() and dist.is_initialized()
    except ImportError:
        ready = False
    if not ready:
        return list(compute(list(params)))
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    mine = shard(len(params), world, rank)
    local = list(compute([params[i] for i in mine])) if len(mine) else []
    if len(local) != len(mine):
        raise RuntimeError("compute returned a wrong number of results")
    gathered = [None] * world
    dist.all_gather_object(gathered, (mine.start, local), group=group)
    out = [None] * len(params)
    for start, res in gathered:
        for k, r in enumerate(res):
            out[start + k] = r
    return out
