"""Replicas: sharding independent chi2 work across processes, one GPU each.

The chi2 pipeline has no exchange step inside it: models (walkers) are
independent, and chi2 is additive over visibility sets.  Work is therefore
spread over processes as replicas, and the only communication is one small
host-side combination of the per-shard results:

- ``ModelShards``: every process holds the whole dataset and evaluates its
  contiguous slice of the B models; the slices' chi2 (and gradients) are
  gathered so that every process sees all B values (what an ensemble sampler
  needs for its next move).
- ``SetShards``: every process holds some of the visibility sets (for example
  spectral windows) and evaluates all B models on them; the per-process chi2
  (B,) and gradients are summed.

Both take an ``evaluate`` callable, so the same logic drives the GPU batched
path (``galario_gb300.batch``) or any other evaluator.  With no initialised
``torch.distributed`` process group they run as a single process.
"""
from __future__ import annotations

from typing import Callable, Optional, Sequence


def shard_bounds(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous balanced partition of range(n): the first n % world shards get one more."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("need 0 <= rank < world")
    if n < 0:
        raise ValueError("n must be non-negative")
    q, r = divmod(n, world)
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def _world(group=None):
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(group), dist.get_world_size(group)
    return 0, 1


def _all_gather_rows(t, n_total: int, world: int, group=None):
    """Gather row blocks of sizes given by shard_bounds(n_total, ., world), in rank order."""
    import torch
    import torch.distributed as dist
    sizes = [shard_bounds(n_total, r, world) for r in range(world)]
    m = max(hi - lo for lo, hi in sizes)
    pad = torch.zeros((m,) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)
    pad[: t.shape[0]] = t
    bufs = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(bufs, pad, group=group)
    return torch.cat([b[: hi - lo] for b, (lo, hi) in zip(bufs, sizes)], dim=0)


class ModelShards:
    """Evaluate B models split across processes.

    evaluate(lo, hi) -> tuple of tensors whose first dimension is hi - lo (the
    chi2 of models lo..hi-1 and, optionally, their gradients).  Returns the
    same tuple for all B models, on every process.
    """

    def __init__(self, evaluate: Callable[[int, int], Sequence], group=None):
        self.evaluate = evaluate
        self.group = group

    def __call__(self, B: int):
        rank, world = _world(self.group)
        lo, hi = shard_bounds(B, rank, world)
        local = self.evaluate(lo, hi)
        single = not isinstance(local, (tuple, list))
        parts = (local,) if single else tuple(local)
        if world == 1:
            return parts[0] if single else parts
        out = tuple(_all_gather_rows(p, B, world, self.group) for p in parts)
        return out[0] if single else out


class SetShards:
    """Evaluate all models on visibility sets split across processes.

    ``sets_of(rank, world)`` is the process's share of the sets (for example
    ``shard_bounds(nsets, rank, world)``); ``evaluate(share)`` returns the
    chi2 (B,) of every model on that share and, optionally, gradients; the
    results are summed over processes (chi2 is additive over sets).
    """

    def __init__(self, evaluate: Callable, sets_of: Optional[Callable] = None, nsets: Optional[int] = None,
                 group=None):
        if sets_of is None:
            if nsets is None:
                raise ValueError("give sets_of or nsets")
            sets_of = lambda r, w: shard_bounds(nsets, r, w)  # noqa: E731
        self.evaluate = evaluate
        self.sets_of = sets_of
        self.group = group

    def __call__(self):
        import torch.distributed as dist
        rank, world = _world(self.group)
        local = self.evaluate(self.sets_of(rank, world))
        single = not isinstance(local, (tuple, list))
        parts = [local] if single else [p.clone() for p in local]
        if single:
            parts = [parts[0].clone()]
        if world > 1:
            for p in parts:
                dist.all_reduce(p, op=dist.ReduceOp.SUM, group=self.group)
        return parts[0] if single else tuple(parts)
