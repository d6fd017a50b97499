"""Corners, Monte-Carlo instances and jobs over several GPUs: replicas only.

One circuit does not shard: a distributed sparse LU would exchange data at
every level of the elimination tree.  Corners, Monte-Carlo instances and
served jobs are independent units, so each rank (one process per GPU) runs a
contiguous share of them on its own device, with no collective on the data
path, and the results are gathered in the original order once, after the
runs (``torch.distributed.all_gather_object``: NCCL between GPU ranks, gloo on
the CPU).  The reference runs its corners one after the other in one process
(vajax/analysis/engine.py:2274-2320, ``run_corners``).
"""

from __future__ import annotations

from typing import Any, Callable, List, Optional, Sequence


def shard(n_items: int, rank: int, world: int) -> range:
    """The contiguous share of ``n_items`` that ``rank`` of ``world`` runs: the
    first ``n_items % world`` ranks take one item more than the others."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} is not in a world of {world}")
    if n_items < 0:
        raise ValueError("n_items must be >= 0")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def run_sharded(items: Sequence[Any], run: Callable[[Any], Any], rank: int = 0, world: int = 1,
                group: Optional[Any] = None) -> List[Any]:
    """Run ``run(item)`` for this rank's share of ``items`` and return every
    rank's results, in the order of ``items``, on every rank."""
    local = [run(items[i]) for i in shard(len(items), rank, world)]
    if world == 1:
        return local
    import torch.distributed as dist
    parts: List[Any] = [None] * world
    dist.all_gather_object(parts, local, group=group)
    return [r for part in parts for r in part]


def run_corners_sharded(engine, corners, rank: int = 0, world: int = 1, group: Optional[Any] = None,
                        **prepare_kwargs):
    """``CircuitEngine.run_corners`` over ``world`` ranks: this rank runs its
    share of ``corners`` in one batched run on its own GPU; the returned sweep
    holds every corner's result, in the order of ``corners``, on every rank."""
    from vajax_gb300.corners import CornerSweepResult
    corners = list(corners)
    mine = [corners[i] for i in shard(len(corners), rank, world)]
    local = engine.run_corners(mine, **prepare_kwargs).results if mine else []
    if world == 1:
        return CornerSweepResult(corners=corners, results=local)
    import torch.distributed as dist
    parts: List[Any] = [None] * world
    dist.all_gather_object(parts, local, group=group)
    return CornerSweepResult(corners=corners, results=[r for part in parts for r in part])
