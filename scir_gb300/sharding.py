"""Channel sharding of a batched-filtering job across ranks (one GPU each).

Every channel is independent (FIR, polyphase resampling and SOS filtering
all act along rows), so N ranks split the rows and run with no data-path
collective.  `shard_rows` gives each rank a contiguous, balanced row range;
`gather_rows` reassembles per-rank results on every rank when a caller wants
one array (it is the only collective, and it is outside the filtering).
"""
from __future__ import annotations


def shard_rows(batch: int, world: int, rank: int) -> tuple[int, int]:
    """Rows [start, stop) of rank `rank` out of `world` (sizes differ by <= 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} not in [0, {world})")
    base, extra = divmod(batch, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def gather_rows(local, batch: int, group=None):
    """All-gathers per-rank row blocks (torch tensors, same trailing shape)
    into one (batch, ...) tensor on every rank."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    sizes = [shard_rows(batch, world, r) for r in range(world)]
    width = max(b - a for a, b in sizes)
    padded = torch.zeros((width,) + tuple(local.shape[1:]), dtype=local.dtype,
                         device=local.device)
    a, b = sizes[rank]
    padded[: b - a] = local
    parts = [torch.empty_like(padded) for _ in range(world)]
    dist.all_gather(parts, padded, group=group)
    return torch.cat([p[: e - s] for p, (s, e) in zip(parts, sizes)], 0)
