"""Launch-shape autotuner for the mixed-precision batch.

The mixed solve places each RVE by a fixed rule: the smallest single CTA or
thread-block cluster (2, 4, then 8 CTAs) whose shared memory holds the RVE's
state. Which cluster sizes pay depends on the GPU and on the size mix: a
cluster trades barrier and distributed-shared-memory costs for on-chip
state, and how many clusters of a size the GPU keeps resident varies. This
tuner times short solves of the batch itself under each limit on the
cluster size (``max_cluster_ctas``) and returns the fastest limit; results
are the same bits under every limit, so only the speed differs.
"""
from __future__ import annotations

import dataclasses
from typing import Dict, Sequence, Tuple

import numpy as np

from .batched import BatchedFiberRVEAnalysisExplicit
from .strategy import SolutionStrategy


def tune_cluster_limit(networks: Sequence, strategies: Sequence, F, steps: int = 100,
                       candidates: Sequence[int] = (1, 2, 4, 8), repeats: int = 2,
                       device: int = 0) -> Tuple[int, Dict[int, float]]:
    """Times `repeats` non-updating solves of `steps` RAMP steps (the
    strategies' damping kept) of the whole batch under each candidate
    cluster-size limit and returns (fastest limit, {limit: fiber-steps/s}).
    F is the (n_rve, 3, 3) deformation gradient of the timed solves."""
    strat = [SolutionStrategy.ramp(steps, s.visc_damp_coeff, s.crit_time_scale_factor)
             for s in strategies]
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(len(networks), 3, 3)
    fiber_steps = float(sum(n.n_fibers for n in networks)) * steps
    table: Dict[int, float] = {}
    for c in candidates:
        g = BatchedFiberRVEAnalysisExplicit(networks, strat, precision="mixed", device=device,
                                            max_cluster_ctas=int(c))
        sigma = np.zeros((len(networks), 6))
        best_ms = None
        for _ in range(repeats + 1):  # the first run captures the launch graph
            g.run(F, sigma, update_coords=False)
            ms, _ = g.last_timing()
            best_ms = ms if best_ms is None else min(best_ms, ms)
        g.close()
        table[int(c)] = fiber_steps / (best_ms * 1e-3)
    best = max(table, key=table.get)
    return best, table
