"""Candidate sharding across GPUs (one process per GPU).

Candidates are independent, so a batch splits into contiguous shards, one per
rank, with the plant tables replicated; no collective touches the data path.
The only exchange is gathering the INFO rows on one rank at the end (the file
API's single INFO_MX_OUT.bin), done with torch.distributed (NCCL across GPUs,
gloo on CPU).
"""
from __future__ import annotations

from typing import Callable

import numpy as np


def shard_bounds(n: int, rank: int, world: int) -> tuple[int, int]:
    """[lo, hi) of rank's contiguous shard; the first n % world ranks get one extra candidate."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} out of range for world size {world}")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def evaluate_sharded(evaluate: Callable[[np.ndarray, np.ndarray], np.ndarray], cuda_mx: np.ndarray,
                     info_in: np.ndarray, group=None, dst: int = 0) -> np.ndarray | None:
    """Evaluate this rank's shard with `evaluate(gains_rows, info_rows) -> info_rows` and
    gather all rows, in candidate order, on rank `dst` (returned there, None elsewhere)."""
    import torch
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    n = cuda_mx.shape[0]
    lo, hi = shard_bounds(n, rank, world)
    out = np.ascontiguousarray(evaluate(cuda_mx[lo:hi], info_in[lo:hi]), np.float32)
    width = info_in.shape[1]
    # pad every shard to the largest so the gather has equal shapes
    rows = -(-n // world)
    buf = torch.zeros((rows, width), dtype=torch.float32)
    buf[:hi - lo] = torch.from_numpy(out)
    backend = dist.get_backend(group)
    if backend == "nccl":
        buf = buf.cuda()
    gathered = [torch.empty_like(buf) for _ in range(world)] if rank == dst else None
    dist.gather(buf, gathered, dst=dst, group=group)
    if rank != dst:
        return None
    parts = []
    for r in range(world):
        a, b = shard_bounds(n, r, world)
        parts.append(gathered[r][:b - a].cpu().numpy())
    return np.vstack(parts)
