"""RVE sharding across GPUs / processes.

RVEs never interact (the reference only distributes them over MPI ranks,
src/mumfim/microscale/MultiscaleRVEAnalysis.cc:102-196), so multi-GPU runs
shard whole RVEs: no collective touches the solve. Work is balanced by
fibers x steps with a greedy longest-processing-time assignment, and results
come back with one all-gather of (rve id, 6 stresses) rows per call.
"""
from __future__ import annotations

import heapq
from typing import List, Sequence

import numpy as np


def shard_rves(work: Sequence[float], world: int) -> List[List[int]]:
    """Assigns RVE ids to `world` ranks, largest work first, each to the
    least-loaded rank (ties to the lower rank). Ids within a shard ascend."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(work)), key=lambda i: (-work[i], i))
    heap = [(0.0, r) for r in range(world)]
    shards: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        heapq.heappush(heap, (load + float(work[i]), r))
    return [sorted(s) for s in shards]


def gather_stress(ids: Sequence[int], sigma: np.ndarray, n_total: int, group=None) -> np.ndarray:
    """All-gathers per-rank stresses (rows of `sigma` belong to RVE `ids`)
    into an (n_total, 6) array on every rank (torch.distributed, any backend)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    n_local = torch.tensor([len(ids)], dtype=torch.int64)
    counts = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(counts, n_local, group=group)
    width = int(max(c.item() for c in counts))
    rows = torch.full((width, 7), float("nan"), dtype=torch.float64)
    if len(ids):
        rows[:len(ids), 0] = torch.tensor(list(ids), dtype=torch.float64)
        rows[:len(ids), 1:] = torch.from_numpy(np.asarray(sigma, dtype=np.float64).reshape(-1, 6))
    parts = [torch.empty_like(rows) for _ in range(world)]
    dist.all_gather(parts, rows, group=group)
    out = np.full((n_total, 6), np.nan)
    for c, p in zip(counts, parts):
        k = int(c.item())
        if k:
            pid = p[:k, 0].numpy().astype(np.int64)
            out[pid] = p[:k, 1:].numpy()
    return out
