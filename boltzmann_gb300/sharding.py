"""Points across GPUs: one process per GPU, each solving its own slice of the points.

The points of a batched 0D3V solve are independent and share only read-only operators
(every rank assembles its own copy of the grid), so the data path has no collective. The
host side needs only a balanced partition of a global batch, the maximum of a time over
ranks (the slowest rank sets the throughput), and a gather of per-point results to rank 0
for output. These use `torch.distributed` on whatever backend the process group has: NCCL
on GPUs, gloo for the host-only tests.
"""
from __future__ import annotations

import numpy as np


def shard_range(n_total: int, rank: int, world: int):
    """(start, count) of rank's contiguous slice of n_total points; the first n_total % world
    ranks take one point more."""
    if world < 1 or not 0 <= rank < world or n_total < 0:
        raise ValueError("bad partition arguments")
    base, extra = divmod(n_total, world)
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def _device():
    import torch
    import torch.distributed as dist
    return torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")


def max_over_ranks(x: float, world: int) -> float:
    """The largest x over the ranks (x itself with one rank)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_points(local: np.ndarray, n_total: int, world: int, axis: int = -1):
    """Concatenate every rank's slice (along `axis`, the point axis) on rank 0 in rank order;
    other ranks get None. Slices may differ in length by one (shard_range)."""
    local = np.ascontiguousarray(local)
    if world == 1:
        return local
    import torch.distributed as dist
    parts = [None] * world if dist.get_rank() == 0 else None
    dist.gather_object(local, parts, dst=0)
    if dist.get_rank() != 0:
        return None
    out = np.concatenate(parts, axis=axis)
    if out.shape[axis] != n_total:
        raise RuntimeError("gathered %d points, expected %d" % (out.shape[axis], n_total))
    return out
