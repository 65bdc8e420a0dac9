"""Several GPUs: (gene set, permutation) units are independent, so each rank
runs its own contiguous range of permutation indices with no collective on
the data path; the only exchange is the host-side gather of the JS values
a set's beta fit needs (main.cu:1488-1497 runs on all R values).

Ranks follow torch.distributed conventions (RANK / WORLD_SIZE); the gather
uses whichever backend the process group was created with (gloo on CPU).
"""
from __future__ import annotations

import numpy as np


def shard(first: int, count: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous split of [first, first+count): (start, length) of `rank`."""
    base, extra = divmod(count, world)
    start = first + rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def gather_values(values: np.ndarray, world: int, dst: int = 0):
    """Concatenates every rank's 1-D float64 array in rank order on `dst`
    (None elsewhere)."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(values, np.float64))
    n = torch.tensor([t.numel()], dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n)
    mx = int(max(s.item() for s in sizes))
    pad = torch.zeros(mx, dtype=torch.float64)
    pad[:t.numel()] = t
    bufs = [torch.zeros(mx, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(bufs, pad)
    if dist.get_rank() != dst:
        return None
    return np.concatenate([b[:int(s.item())].numpy() for b, s in zip(bufs, sizes)])


def sharded_permutation_test(compute, R: int, world: int, rank: int):
    """Iteration 0 on rank 0, iterations 1..R-1 split across ranks;
    compute(first, count) -> (js, U) for this rank's range.  Returns all R JS
    values on rank 0 (None on the others)."""
    start, cnt = shard(1, R - 1, world, rank)
    parts = []
    if rank == 0:
        js0, _ = compute(0, 1)
        parts.append(np.asarray(js0, np.float64))
    if cnt > 0:
        js, _ = compute(start, cnt)
        parts.append(np.asarray(js, np.float64))
    local = np.concatenate(parts) if parts else np.zeros(0)
    return gather_values(local, world)
