"""Host-side logic for running the path on several GPUs, one process each.

Pairs are independent, so several GPUs need no data-path collective.
- A batch is split across ranks by greedy longest-processing-time assignment
  of pairs by cell count. Every rank gets about the same number of cells.
- Each rank runs its shard through the C ABI on its own GPU.
- Rank 0 gathers the result tables on the host.
- Timing takes the maximum over ranks.

The benchmark runs N replicas of one workload (weak scaling) and uses only
``max_over_ranks``. The sharding and gathering serve callers that spread one
large batch over a node's GPUs. All three work on any torch.distributed
backend (``gloo`` on the host, ``nccl`` between GPUs).
"""
from __future__ import annotations

import heapq

import numpy as np


def lpt_shards(cells, world: int) -> list[np.ndarray]:
    """Greedy longest-processing-time assignment of items (pairs) to `world`
    ranks by cost (cells): largest first, each to the least-loaded rank (ties
    to the lowest rank).  Returns each rank's item indices in ascending order.
    The result depends only on the costs, so every rank computes the same
    split without communicating."""
    cells = np.asarray(cells, dtype=np.int64)
    if world < 1:
        raise ValueError("world must be >= 1")
    order = np.argsort(-cells, kind="stable")
    heap = [(0, r) for r in range(world)]
    owner = np.empty(len(cells), dtype=np.int32)
    for k in order:
        load, r = heapq.heappop(heap)
        owner[k] = r
        heapq.heappush(heap, (load + int(cells[k]), r))
    return [np.flatnonzero(owner == r) for r in range(world)]


def max_over_ranks(value: float, group=None) -> float:
    """The largest of each rank's value (the job's time is its slowest
    rank's).  Single process: the value itself."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return float(value)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def gather_table(local: np.ndarray, indices: np.ndarray, n: int, dst: int = 0, group=None):
    """Gathers each rank's result rows (structured array, one row per index
    of its shard) into one table of n rows on rank `dst`; other ranks get
    None.  Host-side; the result rows travel as pickled numpy arrays."""
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        out = np.zeros(n, dtype=local.dtype)
        out[indices] = local
        return out
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    parts = [None] * world if rank == dst else None
    dist.gather_object((indices, local), parts, dst=dst, group=group)
    if rank != dst:
        return None
    out = np.zeros(n, dtype=local.dtype)
    seen = np.zeros(n, dtype=bool)
    for idx, rows in parts:
        if seen[idx].any():
            raise ValueError("shards overlap")
        seen[idx] = True
        out[idx] = rows
    if not seen.all():
        raise ValueError("shards do not cover every pair")
    return out
