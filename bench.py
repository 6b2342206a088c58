"""Benchmark of the batched explicit fiber-network RVE solve.

Default workload (N = 1): config 2, the uneven batch -- 4096 RVEs with node
counts log-uniform in [500, 20000], kNN k in {3, 4, 5} (~52 M fibers), linear
law, F = I + U(+-0.08), 5,000 explicit steps per solve (RAMP protocol: the
boundary follows F linearly over the solve), mixed precision. One bench step
is one batched solve of the whole workload through the C ABI of
libmumfim_gpu.so. Metric: fiber-steps/s = sum over RVEs of fibers x steps,
divided by wall time; RVE solves/s is reported beside it.

  value     inputs resident in HBM, K solves enqueued back to back on one
            stream, CUDA events around them
  e2e       the same solves through mfg_batch_run() with host buffers: per
            step the host->device copy of the deformation gradients and the
            device->host copy of stresses and per-RVE status are inside the
            timed region
  f64_same_batch  the plain FP64 kernel and the mixed kernel on the same
            stratified subset of the batch (every 4th RVE): their throughput
            ratio and the mixed stress error against FP64
  stiffness the FD material stiffness (six perturbed solves) on every 16th
            RVE, mixed precision: the reference's sequential order against
            all six solves in flight at once (the same bits in RAMP mode)
  served_config2  config 2 itself through the continuous-batching server:
            every RVE one request (its F, 5,000 steps), Poisson arrivals at
            80 % of the server's saturated throughput on the same requests;
            throughput over the FP64 kernel's on config 2, p50/p99 latency,
            and the stress error against the FP64 results of f64_same_batch
  config3   the nonlinear-law configuration (2048 RVEs, 20,000 steps): mixed
            throughput on all of it, FP64 on every 8th RVE, the mixed stress
            error overall and binned by the fraction of an RVE's fibers that
            end within 0.01 of the toe's transition stretch
  served_config4  the serving stream at its full 20,000 integration points
            (linear / nonlinear 50/50), load steps x 3 Newton iterations of
            increments I + U(+-0.005), 500 steps per request, Poisson arrivals
            at 80 % of saturation, admission against free HBM; p50/p99 and the
            stress error of a replayed subset against FP64
  roofline  the relaxation kernel's algorithmic bytes (per fiber-step
            20 B + 104 B per node for mixed, 24 B + 108 B per node for FP64)
            over its CUDA-event duration, against the measured HBM bandwidth
            (a model: the state stays on chip); roofline_binding gives the
            resource that does bind, the L1TEX (shared memory) pipe and the
            issue slots, from the committed ncu captures
  autotune  before the timed runs the launch-shape tuner times 500-step
            solves of 1024 RVEs of the batch (stratified by size) under
            every candidate shape -- largest cluster, clusters of 4 instead
            of 2, one or two small RVEs per CTA -- and the batch runs the
            fastest (config.autotune holds the table; every shape gives the
            same bits)
  cpu_baseline  the CPU oracle (a restatement of the reference's batched
            path: the reference itself needs Kokkos, PUMI, AMSI and MPI and
            cannot be built), its optimised timing build, on all host cores,
            on the first RVEs of the batch

``--impl reference`` times only that CPU restatement on the same workload,
with the network generator taken from the oracle's build directory, so that
arm maps no library of the product.
Multi-GPU (torchrun): RVEs are independent; every rank solves its own batch
of the same shape (weak scaling), no collective touches the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

L2_BYTES = 129 * 2**20


def _peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = []
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 8:
                    rows.append(parts)
        os.remove(self.path)
        if not rows:
            return None

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[0]) for r in rows if num(r[0]) is not None]
        mx = [num(r[1]) for r in rows if num(r[1]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def build_workload(config: int, rank: int, n_rve: int | None, solve_steps: int | None = None,
                   nodes: str | None = None):
    from mumfim_gb300 import synthetic as S
    kw = {"steps": solve_steps} if solve_steps else {}
    if nodes:
        if config != 2:
            raise SystemExit("--nodes applies to config 2")
        lo, hi = (int(v) for v in nodes.split(":"))
        kw.update(n_min=lo, n_max=hi)
    if config == 1:
        n = n_rve or 1024
        w = S.config1(n_rve=n, first=rank * n, **kw)
        desc = f"config1: {n} RVEs x 4500 nodes, kNN k=4, linear law, {w.steps} ramp steps"
    elif config == 2:
        n = n_rve or 4096
        w = S.config2(n_rve=n, first=rank * n, **kw)
        band = f"[{kw.get('n_min', 500)},{kw.get('n_max', 20000)}]"
        desc = (f"config2: {n} RVEs, nodes log-uniform {band}, k in {{3,4,5}}, linear law, "
                f"F = I + U(+-0.08), {w.steps} ramp steps")
    elif config == 3:
        n = n_rve or 2048
        w = S.config3(n_rve=n, first=rank * n, **kw)
        desc = f"config3: {n} RVEs, nodes log-uniform [2000,8000], nonlinear law, {w.steps} ramp steps"
    else:
        raise SystemExit("unknown --config")
    return w, desc


def algorithmic_bytes(w, precision: str) -> float:
    """Bytes per solve from the per-fiber-step model: FP64 moves 24 B per fiber
    (connectivity, reference length, two CSR incidences) and 108 B per node
    (x and v read+write, mass, row pointer) every step; mixed moves 20 B per
    fiber and 104 B per node."""
    bf, bn = (24.0, 108.0) if precision == "f64" else (20.0, 104.0)
    return float(w.steps) * (bf * w.total_fibers + bn * w.total_nodes)


def rel_err(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / np.abs(b).max())


def _timing_build_desc():
    from oracle import pyoracle
    return "g++ " + " ".join(pyoracle.timing_flags())


def cpu_baseline(w, sample_rves: int, threads: int):
    from oracle import pyoracle
    sub = w.subset(range(min(sample_rves, w.n_rve)))
    b = pyoracle.OracleBatch(sub.networks, sub.strategies, timing=True)
    t0 = time.perf_counter()
    b.run(sub.F, update_coords=False, n_threads=threads)
    dt = time.perf_counter() - t0
    fs = sub.total_fibers * sub.steps
    return {"value": fs / dt, "unit": "fiber-steps/s", "cores": threads, "kind": "port",
            "sample": f"first {sub.n_rve} RVEs of the workload x {sub.steps} steps "
                      f"({fs:.3g} fiber-steps, {dt:.1f} s; oracle = C++ restatement of the "
                      f"reference's batched path, timing build {_timing_build_desc()}, one RVE "
                      f"per thread, {threads} threads)",
            "rve_solves_per_s": sub.n_rve / dt}


def run_reference(args, rank, world):
    """CPU restatement of the reference path on the host cores (rank 0 only)."""
    if rank != 0:
        return
    from mumfim_gb300 import synthetic as S
    from oracle import pyoracle
    S.use_netgen_library(pyoracle.build_netgen())
    w, desc = build_workload(args.config, 0, args.n_rve, args.solve_steps, args.nodes)
    threads = os.cpu_count() or 1
    sub = w.subset(range(min(args.cpu_sample_rves, w.n_rve)))
    b = pyoracle.OracleBatch(sub.networks, sub.strategies, timing=True)
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        b.run(sub.F, update_coords=False, n_threads=threads)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    fs = sub.total_fibers * sub.steps
    tot = sum(times)
    value = fs * len(times) / tot
    line = {
        "impl": "reference", "metric": "fiber-steps/s", "value": value, "unit": "fiber-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded kNN fiber networks)",
        "config": {"workload": desc, "sample_rves": sub.n_rve, "precision": "f64"},
        "cpu_baseline": {"value": value, "unit": "fiber-steps/s", "cores": threads, "kind": "port",
                         "sample": f"first {sub.n_rve} RVEs x {sub.steps} steps per step; oracle "
                                   f"timing build {_timing_build_desc()}, one RVE per thread"},
        "e2e": {"value": value, "unit": "fiber-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "rve_solves_per_s": sub.n_rve * len(times) / tot,
    }
    print(json.dumps(line), flush=True)


def f64_same_batch(m, w, every: int):
    """Plain FP64 and mixed kernels on the same stratified subset (one solve
    each; the relaxation kernel's CUDA-event time). Returns the summary and
    the subset's ids with its FP64 stresses (the served stream's check)."""
    ids = list(range(0, w.n_rve, every))
    sub = w.subset(ids)
    out = {}
    sig = {}
    for prec in ("f64", "mixed"):
        g = m.BatchedFiberRVEAnalysisExplicit(sub.networks, sub.strategies, precision=prec)
        s = np.zeros((sub.n_rve, 6))
        g.run(sub.F, s, update_coords=False)
        relax_ms, _ = g.last_timing()
        out[prec] = sub.total_fibers * sub.steps / (relax_ms * 1e-3)
        sig[prec] = s.copy()
        g.close()
    summary = {"subset": f"every {every}th RVE ({sub.n_rve} RVEs, {sub.total_fibers} fibers)",
               "f64_fiber_steps_per_s": out["f64"], "mixed_fiber_steps_per_s": out["mixed"],
               "mixed_over_f64": out["mixed"] / out["f64"],
               "sigma_rel_err_mixed_vs_f64": rel_err(sig["mixed"], sig["f64"])}
    return summary, ids, sig["f64"]


def stiffness_section(m, w, every: int):
    """The FD material stiffness on every `every`-th RVE of the batch, mixed
    precision, after an updating solve: the six perturbed solves one after
    the other (the reference's order) and all six in flight at once. In RAMP
    mode both give the same bits; the second of two stiffness calls is
    timed (the first captures the launch graphs)."""
    sub = w.subset(range(0, w.n_rve, every))
    secs, C = {}, {}
    for mode in ("sequential", "concurrent"):
        g = m.BatchedFiberRVEAnalysisExplicit(sub.networks, sub.strategies, precision="mixed",
                                              stiffness=mode)
        g.run(sub.F, update_coords=True)
        g.computeMaterialStiffness()
        t0 = time.perf_counter()
        C[mode] = g.computeMaterialStiffness()
        secs[mode] = time.perf_counter() - t0
        g.close()
    fs = 6.0 * sub.total_fibers * sub.steps
    return {"subset": f"every {every}th RVE ({sub.n_rve} RVEs), {sub.steps} ramp steps per solve",
            "sequential_s": secs["sequential"], "concurrent_s": secs["concurrent"],
            "concurrent_speedup": secs["sequential"] / secs["concurrent"],
            "concurrent_fiber_steps_per_s": fs / secs["concurrent"],
            "bit_identical": bool(np.array_equal(C["sequential"], C["concurrent"]))}


def serve_stream(m, w, passes, update: bool, rate_frac: float = 0.8):
    """Runs `passes` (each a list of per-point F) through one server: first
    one saturation pass of the first pass's requests, all queued at once
    with update_coords = 0 (in RAMP mode a non-updating solve leaves the
    state the next solve starts from unchanged), then every pass as a
    Poisson stream at rate_frac of that throughput. Returns timings,
    latencies and the stream's stresses per pass."""
    from mumfim_gb300 import synthetic as S
    from mumfim_gb300.serving import RVEServer
    n = w.n_rve
    t_create = time.perf_counter()
    sv = RVEServer(w.networks, w.strategies, precision="mixed")
    create_s = time.perf_counter() - t_create
    try:
        t0 = time.perf_counter()
        for p in range(n):
            sv.submit(p, passes[0][p], update_coords=False)
        done = 0
        while done < n:
            done += len(sv.poll(timeout_ms=50))
        sat_s = time.perf_counter() - t0
        rate = rate_frac * n / sat_s
        lat, dev = [], []
        sigma = [np.zeros((n, 6)) for _ in passes]
        status_ok = True
        t_start = time.perf_counter()
        for k, Fk in enumerate(passes):
            arrivals = S.poisson_arrivals(1000 + k, n, rate)
            order = np.argsort(S.uniform(7 + k, n))
            t0 = time.perf_counter()
            i = pending = 0
            while i < n or pending > 0:
                now = time.perf_counter() - t0
                while i < n and arrivals[i] <= now:
                    p = int(order[i])
                    sv.submit(p, Fk[p], update_coords=update)
                    i += 1
                    pending += 1
                res = sv.poll(timeout_ms=0 if i < n else 50)
                pending -= len(res)
                lat.extend(res["latency_s"].tolist())
                dev.extend(res["device_s"].tolist())
                if len(res):
                    sigma[k][res["rve"]] = res["sigma"]
                    status_ok = status_ok and bool((res["status"] == 0).all())
                if i < n:
                    time.sleep(min(max(arrivals[i] - (time.perf_counter() - t0), 0), 0.0005))
        wall = time.perf_counter() - t_start
        launches = sv.launches()
    finally:
        sv.close()
    lat = np.array(lat)
    return {"create_s": create_s, "saturated_rve_solves_per_s": n / sat_s,
            "offered_rate_per_s": rate, "requests": int(len(lat)), "wall_s": wall,
            "latency_p50_ms": float(np.percentile(lat, 50) * 1e3),
            "latency_p99_ms": float(np.percentile(lat, 99) * 1e3),
            "device_p50_ms": float(np.percentile(dev, 50) * 1e3),
            "kernel_launches": int(launches), "all_ok": status_ok}, sigma


def served_config2(m, w, f64_ids, f64_sigma, f64_rate):
    """Config 2 itself as a served stream: one request per RVE (its F, the
    batch's 5,000 steps, update_coords = 0, the same work as a bench step),
    against the FP64 kernel's rate and stresses on the same batch."""
    r, sigma = serve_stream(m, w, [list(w.F)], update=False)
    fs = float(w.total_fibers) * w.steps
    r["fiber_steps_per_s"] = fs / r["wall_s"]
    r["rve_solves_per_s"] = w.n_rve / r["wall_s"]
    r["served_over_f64"] = r["fiber_steps_per_s"] / f64_rate
    r["sigma_rel_err_vs_f64"] = rel_err(sigma[0][f64_ids], f64_sigma)
    r["workload"] = (f"config2: all {w.n_rve} RVEs, one request each ({w.steps} ramp steps), "
                     f"Poisson arrivals at 80 % of the server's saturated throughput; FP64 "
                     f"rate and stresses from f64_same_batch ({len(f64_ids)} RVEs of the batch)")
    return r


def served_config4(m, n_points: int, load_steps: int, iters: int, steps: int, check: int):
    """The config-4 serving stream: n_points persistent RVEs, load_steps x
    iters updating increments per point, Poisson arrivals at 80 % of
    saturation; the first `check` points replayed on the FP64 kernel."""
    from mumfim_gb300 import synthetic as S
    t0 = time.perf_counter()
    w = S.config4(n_points=n_points, steps=steps)
    gen_s = time.perf_counter() - t0
    passes = [[S.config4_increment(p, ls, it) for p in range(n_points)]
              for ls in range(load_steps) for it in range(iters)]
    r, sigma = serve_stream(m, w, passes, update=True)
    fs = float(w.total_fibers) * steps * len(passes)
    r["fiber_steps_per_s"] = fs / r["wall_s"]
    r["rve_solves_per_s"] = r["requests"] / r["wall_s"]
    sub = w.subset(range(check))
    g = m.BatchedFiberRVEAnalysisExplicit(sub.networks, sub.strategies, precision="f64")
    errs = []
    for k, Fk in enumerate(passes):
        s = np.zeros((check, 6))
        g.run(np.stack(Fk[:check]), s, update_coords=True)
        errs.append(rel_err(sigma[k][:check], s))
    g.close()
    r["sigma_rel_err_vs_f64"] = float(max(errs))
    r["checked_points"] = check
    r["generate_s"] = gen_s
    r["workload"] = (f"config4: {n_points} persistent RVEs (integration points), nodes log-uniform "
                     f"[500,20000], k in {{3,4,5}}, linear/nonlinear 50/50, {load_steps} load "
                     f"steps x {iters} Newton iterations (of the configuration's 50 x 3), "
                     f"increments I + U(+-0.005), {steps} ramp steps per request, Poisson "
                     f"arrivals at 80 % of saturation, admission against free HBM")
    return r


def config3_section(m, every: int):
    """Config 3 as specified: mixed throughput on the whole batch, FP64 on
    every `every`-th RVE, and the mixed stress error against FP64 -- overall
    and by how many of an RVE's fibers end near the toe's transition stretch
    (|lambda - lambda_t| <= 0.01, lambda from the FP64 solve's final
    coordinates)."""
    from mumfim_gb300 import synthetic as S
    w = S.config3()
    g = m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision="mixed")
    s_all = np.zeros((w.n_rve, 6))
    g.run(w.F, s_all, update_coords=False)
    mixed_ms, _ = g.last_timing()
    g.close()
    ids = list(range(0, w.n_rve, every))
    sub = w.subset(ids)
    g = m.BatchedFiberRVEAnalysisExplicit(sub.networks, sub.strategies, precision="f64")
    s64 = np.zeros((sub.n_rve, 6))
    g.run(sub.F, s64, update_coords=False)
    f64_ms, _ = g.last_timing()
    near = np.zeros(sub.n_rve)
    for r, net in enumerate(sub.networks):
        x = g.coordinates(r)
        c = net.connectivity
        lam = (np.linalg.norm(x[c[:, 1]] - x[c[:, 0]], axis=1)
               / np.linalg.norm(net.coords[c[:, 1]] - net.coords[c[:, 0]], axis=1))
        near[r] = float(np.mean(np.abs(lam - net.reactions[0].length_ratio_trns) <= 0.01))
    g.close()
    sm = s_all[ids]
    err = np.abs(sm - s64).max(axis=1) / np.abs(s64).max(axis=1)
    q = np.quantile(near, [0.0, 0.25, 0.5, 0.75, 1.0])
    bins = []
    for lo, hi in zip(q[:-1], q[1:]):
        sel = (near >= lo) & (near <= hi)
        bins.append({"near_toe_frac": [float(lo), float(hi)], "rves": int(sel.sum()),
                     "max_rel_err": float(err[sel].max())})
    return {"workload": f"config3: {w.n_rve} RVEs, nodes log-uniform [2000,8000], "
                        f"exponential-toe law, {w.steps} ramp steps",
            "mixed_fiber_steps_per_s": w.total_fibers * w.steps / (mixed_ms * 1e-3),
            "f64_fiber_steps_per_s": sub.total_fibers * sub.steps / (f64_ms * 1e-3),
            "f64_subset": f"every {every}th RVE ({sub.n_rve} RVEs; fewer RVEs than the FP64 "
                          f"kernel's resident CTAs, so its rate is a lower bound -- "
                          f"f64_same_batch has the full-occupancy FP64 rate)",
            "sigma_rel_err_mixed_vs_f64": float(err.max()),
            "sigma_rel_err_median": float(np.median(err)),
            "rves_over_1e-5": int((err > 1e-5).sum()),
            "worst_rve": int(ids[int(np.argmax(err))]),
            "near_toe_frac_mean": float(near.mean()),
            "err_by_near_toe_quartile": bins}


def roofline_binding():
    """Time-weighted L1TEX pipe and issue-slot fractions of the mixed
    kernel's size buckets, from the committed ncu captures."""
    p = os.path.join(REPO, "profiles", "binding_config2_mixed.json")
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        d = json.load(fh)
    b = d["buckets"]
    tot = sum(v["time_share"] for v in b.values())
    l1 = sum(v["time_share"] * v["l1tex_pipe_frac"] for v in b.values()) / tot
    iss = sum(v["time_share"] * v["issue_slots_frac"] for v in b.values()) / tot
    return {"resource": "L1TEX pipe (shared and distributed shared memory)", "frac": l1,
            "issue_slots_frac": iss, "unit": "fraction of peak, ncu, time-weighted over buckets",
            "source": "profiles/binding_config2_mixed.json"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=2)
    ap.add_argument("--n-rve", type=int, default=None)
    ap.add_argument("--precision", default="mixed", choices=["f64", "mixed"])
    ap.add_argument("--cpu-sample-rves", type=int, default=64)
    ap.add_argument("--solve-steps", type=int, default=None,
                    help="override the explicit steps per solve (small profiling cases)")
    ap.add_argument("--nodes", default=None, metavar="LO:HI",
                    help="config 2 with node counts log-uniform in [LO, HI] (profiling cases)")
    ap.add_argument("--f64-every", type=int, default=4)
    ap.add_argument("--serve-points", type=int, default=20_000,
                    help="integration points of the config-4 stream")
    ap.add_argument("--serve-load-steps", type=int, default=1,
                    help="load steps of the config-4 stream (3 Newton iterations each)")
    ap.add_argument("--serve-steps", type=int, default=500)
    ap.add_argument("--config3-every", type=int, default=8)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--small-rve-solve", choices=("auto", "node", "fiber"), default="auto",
                    help="mixed: solve of the RVEs whose node state fits one CTA "
                         "(auto = node-centric)")
    ap.add_argument("--small-rves-per-cta", type=int, default=0,
                    help="mixed, fiber-centric small solve: small RVEs side by side per CTA "
                         "(1 or 2; 0 = 2)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="mixed: skip the launch-shape tuner (mumfim_gb300.autotune) and use "
                         "the default shape")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the FP64 side-by-side, the served streams and config 3")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")

    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch
    torch.cuda.set_device(local_rank)
    import mumfim_gb300 as m

    w, desc = build_workload(args.config, rank, args.n_rve, args.solve_steps, args.nodes)
    tune = None
    shape = {"small_rves_per_cta": args.small_rves_per_cta, "small_rve_solve": args.small_rve_solve}
    if (args.precision == "mixed" and not args.no_autotune and not args.small_rves_per_cta
            and args.small_rve_solve == "auto"):
        import dataclasses

        from mumfim_gb300.autotune import tune_launch_shape
        best, rep = tune_launch_shape(w.networks, w.strategies, w.F, device=local_rank)
        shape = best.kwargs()
        tune = {"best": dataclasses.asdict(best), "from_cache": rep["from_cache"],
                "seconds": rep["seconds"], "sample_rves": rep["sample_rves"],
                "steps": rep["steps"], "table": rep["table"]}
    t0 = time.perf_counter()
    gpu = m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision=args.precision,
                                            device=local_rank, **shape)
    setup_s = time.perf_counter() - t0
    R = w.n_rve
    fiber_steps = w.total_fibers * w.steps
    dev = torch.device("cuda", local_rank)
    # A dedicated (non-default) stream: the library launches on it and the
    # CUDA events below are recorded on it.
    stream = torch.cuda.Stream(dev)
    with torch.cuda.stream(stream):
        F_dev = torch.from_numpy(np.ascontiguousarray(w.F.reshape(R, 9))).to(dev)
        sig_dev = torch.zeros((R, 6), dtype=torch.float64, device=dev)
        st_dev = torch.zeros((R, 2), dtype=torch.float64, device=dev)  # 16-byte status records
    stream.synchronize()

    def device_step():
        gpu.run_device(F_dev.data_ptr(), R, sig_dev.data_ptr(), update_coords=False,
                       status_ptr=st_dev.data_ptr(), stream=stream.cuda_stream)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()

    # ---- value: device-resident inputs ----------------------------------
    for _ in range(args.warmup):
        device_step()
    barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    barrier()
    ev[0].record(stream)
    for k in range(args.steps):
        device_step()
        ev[k + 1].record(stream)
    ev[-1].synchronize()
    barrier()
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    t_ms = sum(step_ms)
    launches_per_step = gpu.last_launches()
    relax_ms, run_ms = gpu.last_timing()
    if dist:
        t = torch.tensor([t_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_ms = float(t.item())
    value = world * fiber_steps * args.steps / (t_ms * 1e-3)

    # ---- e2e: host buffers through mfg_batch_run -----------------------------
    F_host = torch.from_numpy(np.ascontiguousarray(w.F.reshape(R, 3, 3))).pin_memory().numpy()
    sig_host = torch.zeros((R, 6), dtype=torch.float64).pin_memory().numpy()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gpu.run(F_host, sig_host, update_coords=False)
    barrier()
    e2e_s = time.perf_counter() - t0
    clk = clocks.stop()
    if dist:
        t = torch.tensor([e2e_s], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = world * fiber_steps * args.steps / e2e_s
    ok_frac = float(np.mean(gpu.last_status["status"] == 0))
    gpu.close()

    # ---- roofline of the relaxation kernel -----------------------------------
    peak, peak_kind = _peaks()
    alg = algorithmic_bytes(w, args.precision)
    achieved = alg / (relax_ms * 1e-3) / 1e9
    traffic = None
    tp = os.path.join(REPO, "profiles", f"traffic_config{args.config}_{args.precision}.json")
    if os.path.exists(tp):
        with open(tp) as fh:
            tr = json.load(fh)
        traffic = tr.get("dram_bytes_per_fiber_step", 0) * fiber_steps or None

    line = {
        "metric": "fiber-steps/s", "value": value, "unit": "fiber-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "f64" else "f32+f64",
        "data": "synthetic (seeded kNN fiber networks; no public dataset for this path)",
        "config": {"workload": desc, "n_rve_per_gpu": R, "fibers_per_gpu": w.total_fibers,
                   "nodes_per_gpu": w.total_nodes, "explicit_steps_per_solve": w.steps,
                   "precision": args.precision, "mode": "ramp (fixed steps, linear boundary F)",
                   "l2": f"working set > L2 ({L2_BYTES >> 20} MiB): no flush needed",
                   "parallelism": f"rve-sharded x{world}", "setup_s": round(setup_s, 2),
                   "autotune": tune},
        "rve_solves_per_s": world * R * args.steps / (t_ms * 1e-3),
        "e2e": {"value": e2e, "unit": "fiber-steps/s", "h2d_bytes_per_step": int(F_host.nbytes),
                "d2h_bytes_per_step": int(sig_host.nbytes + 16 * R)},
        "gpu_launches": int(launches_per_step * args.steps),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": f"{peak_kind} hbm_gbs (burst)",
                     "kernel": "relax_f64_kernel" if args.precision == "f64" else "relax_mixed_kernel",
                     "kernel_ms": relax_ms},
        "converged_or_completed_frac": ok_frac,
    }
    if clk:
        line["clocks"] = clk
    binding = roofline_binding() if args.precision == "mixed" else None
    if binding:
        line["roofline_binding"] = binding
    if rank == 0 and world == 1 and not args.no_extras:
        summary, ids, s64 = f64_same_batch(m, w, args.f64_every)
        line["f64_same_batch"] = summary
        if args.precision == "mixed":
            line["stiffness"] = stiffness_section(m, w, 16)
        if args.config == 2 and args.precision == "mixed":
            line["served_config2"] = served_config2(m, w, ids, s64,
                                                    summary["f64_fiber_steps_per_s"])
        line["config3"] = config3_section(m, args.config3_every)
        line["served_config4"] = served_config4(m, args.serve_points, args.serve_load_steps, 3,
                                                args.serve_steps, 32)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, args.cpu_sample_rves, os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
