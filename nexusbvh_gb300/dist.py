"""Host-side multi-GPU helpers: one process per GPU, no collective on the data path.

A single mesh does not shard (its scene box and global sort would need an
all-reduce and an all-to-all, and H-PLOC's top merges cross any partition),
so plain builds run as replicas.  Batched and served work shards by whole
mesh: each rank builds a disjoint subset of the meshes with its own batch,
and the only collective is the max of the ranks' timings used to report
whole-job throughput.
"""
from __future__ import annotations

import heapq

import numpy as np


def shard_meshes(counts, world: int, rank: int) -> np.ndarray:
    """Indices of the meshes rank `rank` builds: largest meshes first, each
    to the rank with the fewest triangles so far (ties to the lower rank), so
    every rank gets a similar triangle count.  Deterministic; the shards are
    disjoint and cover every mesh."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    counts = np.asarray(counts, dtype=np.int64)
    order = np.lexsort((np.arange(len(counts)), -counts))  # by size desc, then index
    heap = [(0, r) for r in range(world)]
    mine = []
    for m in order:
        load, r = heapq.heappop(heap)
        if r == rank:
            mine.append(int(m))
        heapq.heappush(heap, (load + int(counts[m]), r))
    return np.array(sorted(mine), dtype=np.int64)


def max_over_ranks(value: float, device=None) -> float:
    """Max of a per-rank float over the process group (value itself if not
    distributed).  Works with gloo (CPU tensors) and NCCL (device tensors)."""
    import torch
    import torch.distributed as td
    if not (td.is_available() and td.is_initialized()) or td.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    """Sum of a per-rank float over the process group (value if not distributed)."""
    import torch
    import torch.distributed as td
    if not (td.is_available() and td.is_initialized()) or td.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    td.all_reduce(t, op=td.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(units_per_rank: float, elapsed_s_per_rank: float, device=None) -> float:
    """Units processed by all ranks divided by the slowest rank's time."""
    units = sum_over_ranks(units_per_rank, device)
    slowest = max_over_ranks(elapsed_s_per_rank, device)
    return units / slowest if slowest > 0 else 0.0
