"""Host logic of multi-GPU runs: one process per GPU, launched by torchrun.

msp on one graph does not shard: every sub-round needs the global frontier
and the support state, so N GPUs run N independent replicas.  Batches of
independent graphs shard by graph: rank r of N takes its own run of graphs
(weak scaling: per-GPU work stays fixed as N grows), and no data-path
collective is needed.  The only collectives are the timing barrier, the
maximum of the timed region over ranks, and (for checks) a gather of small
per-rank summaries.
"""

from __future__ import annotations

import os


def dist_env() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def batch_shard(per_rank: int, rank: int, total: int | None = None) -> list[int]:
    """Graph indices of rank `rank` when every rank decomposes `per_rank`
    graphs of the batch: the run [rank * per_rank, (rank + 1) * per_rank),
    clipped to `total` graphs when given."""
    lo = rank * per_rank
    hi = lo + per_rank
    if total is not None:
        lo, hi = min(lo, total), min(hi, total)
    return list(range(lo, hi))


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of `value` over the ranks of the default process group (the
    value itself without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier() -> None:
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def gather(obj) -> list:
    """Every rank's `obj` (a small picklable summary), in rank order."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [obj]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out
