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


# fields of pecs_params that define the meshes and the fixed matrices: points
# that agree on them can share a context (validate_params checks the same set)
MATRIX_FIELDS = ("degree", "full_system", "nx_semi", "nx_elec", "ny", "x_semi0", "x_semi1", "x_elec1",
                 "height", "lambda2", "eps_semi", "eps_elec", "mu", "dt", "penalty", "bc_semi",
                 "bc_elec", "bc_poisson", "grading", "bc_poisson_elec", "poisson_pairing")


def matrix_key(p) -> tuple:
    return tuple(tuple(v) if isinstance(v, (list, tuple)) else v for v in
                 (getattr(p, f) for f in MATRIX_FIELDS))


def ragged_sweep(points: Sequence, slots: int = 64, precision: int = None, max_steps: int = 5000,
                 tol: float = 1e-8, check_every: int = 50, want_fields: bool = False,
                 concurrent: bool = False, **ctx_kw):
    """I-V points of uneven size (different refinement levels, degrees or other
    matrix-defining parameters) to steady state: the points are grouped by
    their meshes and fixed matrices, and each group is streamed through one
    context of at most ``slots`` slots (pecs_sweep_stream).  Results come back
    in the order of ``points``: (steps, currents, fields or None), fields as
    one array per point and field.

    ``concurrent``: every group's context is created first (one after
    another: setup uses all host threads), then the groups' sweeps run at the
    same time, one host thread per group, each on its context's own CUDA
    stream, so that small meshes fill the SMs a large mesh leaves idle.  The
    results are those of the groups run one after another: each context's
    kernels and step sequence are the same either way."""
    import numpy as np

    from .api import PREC_FP64, Context
    prec = PREC_FP64 if precision is None else precision
    groups = {}
    for i, p in enumerate(points):
        groups.setdefault(matrix_key(p), []).append(i)
    steps = np.zeros(len(points), dtype=np.int64)
    cur = np.zeros(len(points))
    fields = [None] * len(points) if want_fields else None

    def finish(idx, ctx, res):
        s, c, fin = res
        for k, i in enumerate(idx):
            steps[i] = s[k]
            cur[i] = c[k]
            if want_fields:
                fields[i] = {f: fin[f][k * ctx.ndofs[f]:(k + 1) * ctx.ndofs[f]].copy() for f in fin}

    def make(idx):
        pts = [points[i] for i in idx]
        return pts, Context(pts[:min(slots, len(pts))], precision=prec, **ctx_kw)

    if not concurrent:
        for idx in groups.values():
            pts, ctx = make(idx)
            try:
                finish(idx, ctx, ctx.sweep_stream(pts, max_steps, tol, check_every, want_fields=want_fields))
            finally:
                ctx.close()
        return steps, cur, fields

    from concurrent.futures import ThreadPoolExecutor
    made = []
    try:
        for idx in groups.values():
            made.append((idx,) + make(idx))
        with ThreadPoolExecutor(max_workers=max(1, len(made))) as pool:
            futs = [pool.submit(ctx.sweep_stream, pts, max_steps, tol, check_every, want_fields=want_fields)
                    for _, pts, ctx in made]
            results = [f.result() for f in futs]
        for (idx, _, ctx), res in zip(made, results):
            finish(idx, ctx, res)
    finally:
        for _, _, ctx in made:
            ctx.close()
    return steps, cur, fields
