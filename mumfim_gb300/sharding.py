"""RVE sharding across GPUs / processes.

RVEs never interact (the reference only distributes them over MPI ranks,
src/mumfim/microscale/MultiscaleRVEAnalysis.cc:102-196), so multi-GPU runs
shard whole RVEs: no collective touches the solve. Work is balanced by
fibers x steps with a greedy longest-processing-time assignment, and results
come back with one all-gather of (rve id, 6 stresses) rows per call.
"""
from __future__ import annotations

import datetime
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


class RankFailure(RuntimeError):
    """A rank did not reach a step within the liveness bound."""

    def __init__(self, message: str, missing: Sequence[int]):
        super().__init__(message)
        self.missing = list(missing)


def await_peers(store, tag: str, rank: int, world: int, timeout_s: float) -> None:
    """Host-side liveness check between steps, before any rank launches the
    next solve: every rank announces `tag` in the key-value store (a
    torch.distributed TCPStore or FileStore) and waits, at most timeout_s, for
    every other rank's announcement. Raises RankFailure naming the ranks that
    did not announce, so the survivors stop cleanly instead of blocking in
    their next collective. The reference has no such check: an MPI rank that
    dies leaves the others in their next collective."""
    store.set(f"{tag}/{rank}", b"1")
    keys = [f"{tag}/{r}" for r in range(world)]
    try:
        store.wait(keys, datetime.timedelta(seconds=timeout_s))
    except Exception as e:
        missing = [r for r in range(world) if not store.check([f"{tag}/{r}"])]
        if not missing:
            raise
        raise RankFailure(f"ranks {missing} did not reach {tag!r} within {timeout_s} s",
                          missing) from e
