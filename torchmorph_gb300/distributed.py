"""Multi-GPU helpers.  The operators are batch-parallel with no exchange step:
every (b, c) item, every ragged image and every OT problem is independent, so
N GPUs each run their own share of the batch and only the host reduces the
timing.  No collective runs on the data path."""

from __future__ import annotations

import torch


def split_batch(n_items: int, rank: int, world: int) -> slice:
    """Contiguous, balanced share of `n_items` for `rank` (sizes differ by at most 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} for world size {world}")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank scalar over the default process group (identity without one)."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())
