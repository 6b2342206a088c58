"""Launch-shape autotuner for the mixed-precision batch.

The mixed solve places each RVE by rule: the smallest single CTA or
thread-block cluster (2, 4, then 8 CTAs) whose shared memory holds the
RVE's node state (node-centric solve), else one CTA streaming from global
memory; on request, RVEs whose whole state fits one CTA (or half of one,
two per CTA) take the fiber-centric solve first. Which shapes pay depends
on the GPU and on the size mix: a cluster trades barrier and
distributed-shared-memory costs for on-chip state, how many clusters of a
size stay resident varies, and the fiber-centric solve of small RVEs trades
half the fiber arithmetic against a stored force vector per fiber and a
second pass. The tuner times short solves of a size-stratified sample of
the batch under every candidate shape -- the largest cluster allowed
(``max_cluster_ctas``), clusters of 4 instead of 2 (the serving layout) and
the solve of small RVEs (node-centric, or fiber-centric two per CTA) -- and
keeps the fastest. Every candidate gives the same bits, so only the speed
differs.

Choices are cached per (GPU, SM count, size-mix histogram, law mix) in a
JSON file (``MFG_AUTOTUNE_CACHE``, default ``mumfim_gb300/_lib/autotune.json``).
"""
from __future__ import annotations

import dataclasses
import json
import os
import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .batched import BatchedFiberRVEAnalysisExplicit
from .strategy import SolutionStrategy

_PKG = os.path.dirname(os.path.abspath(__file__))


@dataclasses.dataclass(frozen=True)
class LaunchShape:
    max_cluster_ctas: int = 0     # 1, 2, 4 or 8 (0 = 8)
    serving_layout: bool = False  # clusters of 4 where the batch layout takes 2
    small_rves_per_cta: int = 0   # fiber-centric small solve: 1 or 2 (0 = 2)
    small_rve_solve: str = "auto"  # "auto" (= "node"), "node" or "fiber"

    def kwargs(self) -> dict:
        return dict(max_cluster_ctas=self.max_cluster_ctas, serving_layout=self.serving_layout,
                    small_rves_per_cta=self.small_rves_per_cta,
                    small_rve_solve=self.small_rve_solve)


DEFAULT_SHAPE = LaunchShape(8, False, 0, "auto")
CANDIDATES_VERSION = 3  # small solve: auto (by law), node- or fiber-centric


def candidate_shapes(nonlinear_frac: float = 0.0) -> List[LaunchShape]:
    """Every distinct shape: the serving layout only differs from the batch
    layout when clusters of 4 are allowed; the small solve "auto" (node-
    centric on the linear law, fiber-centric on the nonlinear one) is tried
    beside whichever of "node" and "fiber" differs from it on this law mix,
    the fiber-centric one with two small RVEs per CTA (one per CTA measured
    slower)."""
    solves = [("auto", 2)]
    if nonlinear_frac > 0.0:
        solves.append(("node", 0))
    if nonlinear_frac < 1.0:
        solves.append(("fiber", 2))
    out = []
    for solve, per_cta in solves:
        for mc in (8, 4, 2, 1):
            out.append(LaunchShape(mc, False, per_cta, solve))
            if mc >= 4:
                out.append(LaunchShape(mc, True, per_cta, solve))
    return out


def stratified_sample(networks: Sequence, size: int) -> List[int]:
    """Ids of at most `size` RVEs spread evenly over the batch sorted by
    node count (so the sample keeps the size mix)."""
    n = len(networks)
    if n <= size:
        return list(range(n))
    order = sorted(range(n), key=lambda r: (networks[r].n_nodes, r))
    return sorted(order[int(i * n / size)] for i in range(size))


def workload_key(networks: Sequence, device: int = 0) -> str:
    """Cache key: GPU name and SM count, the histogram of log2(node count) in
    half-octave bins (fractions to 0.02), mean fibers per node, the
    fraction of RVEs on the nonlinear law, and the version of the candidate
    set (a choice among other candidates is not reused)."""
    try:
        import torch
        p = torch.cuda.get_device_properties(device)
        gpu = f"{p.name}|{p.multi_processor_count}"
    except Exception:
        gpu = "unknown"
    nodes = np.array([n.n_nodes for n in networks], dtype=np.float64)
    bins = np.round(2 * np.log2(nodes)).astype(int)
    vals, counts = np.unique(bins, return_counts=True)
    hist = {int(v): round(float(c) / len(nodes) / 0.02) * 0.02 for v, c in zip(vals, counts)}
    hist = {k: round(v, 2) for k, v in hist.items() if v > 0}
    fpn = round(float(sum(n.n_fibers for n in networks)) / float(nodes.sum()), 1)
    nl = round(float(np.mean([n.reactions[0].law == 1 for n in networks])), 1)
    return json.dumps({"gpu": gpu, "hist": hist, "fibers_per_node": fpn, "nonlinear": nl,
                       "candidates": CANDIDATES_VERSION}, sort_keys=True)


def _cache_path() -> str:
    return os.environ.get("MFG_AUTOTUNE_CACHE", os.path.join(_PKG, "_lib", "autotune.json"))


def _load_cache() -> dict:
    try:
        with open(_cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store_cache(key: str, entry: dict) -> None:
    c = _load_cache()
    c[key] = entry
    path = _cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(c, fh, indent=1)
    os.replace(tmp, path)


def _rate(networks, strat, F, shape: LaunchShape, repeats: int, device: int) -> float:
    g = BatchedFiberRVEAnalysisExplicit(networks, strat, precision="mixed", device=device,
                                        **shape.kwargs())
    sigma = np.zeros((len(networks), 6))
    best_ms = None
    for _ in range(repeats + 1):  # the first run captures the launch graph
        g.run(F, sigma, update_coords=False)
        ms, _ = g.last_timing()
        best_ms = ms if best_ms is None else min(best_ms, ms)
    g.close()
    steps = strat[0].max_steps
    return float(sum(n.n_fibers for n in networks)) * steps / (best_ms * 1e-3)


def tune_launch_shape(networks: Sequence, strategies: Sequence, F, steps: int = 500,
                      sample: int = 1024, repeats: int = 2, device: int = 0,
                      candidates: Optional[Sequence[LaunchShape]] = None,
                      use_cache: bool = True) -> Tuple[LaunchShape, dict]:
    """Returns (fastest shape, report). The report holds the cache key, where
    the choice came from, and the table of fiber-steps/s per candidate shape
    (timed on `sample` RVEs of the batch, `steps` RAMP steps, non-updating,
    best of `repeats` solves)."""
    key = workload_key(networks, device)
    if use_cache:
        hit = _load_cache().get(key)
        if hit:
            return LaunchShape(**hit["best"]), dict(hit, from_cache=True, key=key)
    t0 = time.perf_counter()
    ids = stratified_sample(networks, sample)
    nets = [networks[r] for r in ids]
    strat = [SolutionStrategy.ramp(steps, strategies[r].visc_damp_coeff,
                                   strategies[r].crit_time_scale_factor) for r in ids]
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(len(networks), 3, 3)[ids]
    table = []
    nl = float(np.mean([n.reactions[0].law == 1 for n in networks]))
    for shape in (candidates or candidate_shapes(nl)):
        table.append({"shape": dataclasses.asdict(shape),
                      "fiber_steps_per_s": _rate(nets, strat, F, shape, repeats, device)})
    best = max(table, key=lambda t: t["fiber_steps_per_s"])
    entry = {"best": best["shape"], "table": table, "sample_rves": len(ids), "steps": steps,
             "seconds": round(time.perf_counter() - t0, 1)}
    if use_cache:
        _store_cache(key, entry)
    return LaunchShape(**best["shape"]), dict(entry, from_cache=False, key=key)


def tune_cluster_limit(networks: Sequence, strategies: Sequence, F, steps: int = 100,
                       candidates: Sequence[int] = (1, 2, 4, 8), repeats: int = 2,
                       device: int = 0) -> Tuple[int, Dict[int, float]]:
    """The cluster-size limit alone, on the whole batch: (fastest limit,
    {limit: fiber-steps/s})."""
    strat = [SolutionStrategy.ramp(steps, s.visc_damp_coeff, s.crit_time_scale_factor)
             for s in strategies]
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(len(networks), 3, 3)
    table = {int(c): _rate(networks, strat, F, LaunchShape(int(c), False, 0), repeats, device)
             for c in candidates}
    return max(table, key=table.get), table
