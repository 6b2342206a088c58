"""Benchmark of the batched explicit fiber-network RVE solve.

One bench step = one batched solve: every RVE of the workload relaxed for the
configured number of explicit steps (RAMP protocol: the boundary follows F
linearly over the solve), through the C ABI of libmumfim_gpu.so.

Default workload (N = 1): config 1 -- 1024 RVEs x 4500 nodes, k = 4
nearest-neighbour fibers (~11,100 fibers each), linear law, 5,000 steps,
plain FP64 kernel. Metric: fiber-steps/s = sum over RVEs of fibers x steps,
divided by wall time; RVE solves/s is reported beside it.

  value     inputs resident in HBM, K solves enqueued back to back on one
            stream, CUDA events around them
  e2e       the same solves through mfg_batch_run() with host buffers: per
            step the host->device copy of the deformation gradients and the
            device->host copy of stresses and per-RVE status are inside the
            timed region
  roofline  the relaxation kernel's algorithmic bytes (per fiber-step
            24 + 108 N/E bytes for FP64, counted from the workload) over its
            CUDA-event duration, against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (a restatement of the reference's batched
            path: the reference itself cannot be built without Kokkos, PUMI,
            AMSI and MPI) on the host's cores, on a bounded subset of RVEs

``--impl reference`` times only that CPU restatement on the same workload.
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


def build_workload(config: int, rank: int, n_rve: int | None, solve_steps: int | None = None):
    from mumfim_gb300 import synthetic as S
    kw = {"steps": solve_steps} if solve_steps else {}
    if config == 1:
        n = n_rve or 1024
        w = S.config1(n_rve=n, first=rank * n, **kw)
        desc = f"config1: {n} RVEs x 4500 nodes, kNN k=4, linear law, {w.steps} ramp steps"
    elif config == 2:
        n = n_rve or 4096
        w = S.config2(n_rve=n, first=rank * n, **kw)
        desc = f"config2: {n} RVEs, nodes log-uniform [500,20000], k in {{3,4,5}}, {w.steps} ramp steps"
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


def cpu_baseline(w, sample_rves: int, threads: int):
    from oracle import pyoracle
    sub = w.subset(range(min(sample_rves, w.n_rve)))
    b = pyoracle.OracleBatch(sub.networks, sub.strategies)
    t0 = time.perf_counter()
    b.run(sub.F, update_coords=False, n_threads=threads)
    dt = time.perf_counter() - t0
    fs = sub.total_fibers * sub.steps
    return {"value": fs / dt, "unit": "fiber-steps/s", "cores": threads, "kind": "port",
            "sample": f"{sub.n_rve} RVEs of the workload x {sub.steps} steps "
                      f"({fs:.3g} fiber-steps, {dt:.1f} s, oracle built -O2 -ffp-contract=off)",
            "rve_solves_per_s": sub.n_rve / dt}


def run_reference(args, rank, world):
    """CPU restatement of the reference path on the host cores (rank 0 only)."""
    if rank != 0:
        return
    w, desc = build_workload(args.config, 0, args.n_rve, args.solve_steps)
    threads = os.cpu_count() or 1
    from oracle import pyoracle
    sub = w.subset(range(min(args.cpu_sample_rves, w.n_rve)))
    b = pyoracle.OracleBatch(sub.networks, sub.strategies)
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
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded kNN networks)",
        "config": {"workload": desc, "sample_rves": sub.n_rve, "precision": "f64"},
        "cpu_baseline": {"value": value, "unit": "fiber-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{sub.n_rve} RVEs x {sub.steps} steps per step"},
        "e2e": {"value": value, "unit": "fiber-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "rve_solves_per_s": sub.n_rve * len(times) / tot,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--n-rve", type=int, default=None)
    ap.add_argument("--precision", default="f64", choices=["f64", "mixed"])
    ap.add_argument("--cpu-sample-rves", type=int, default=48)
    ap.add_argument("--solve-steps", type=int, default=None,
                    help="override the explicit steps per solve (small profiling cases)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
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

    w, desc = build_workload(args.config, rank, args.n_rve, args.solve_steps)
    t0 = time.perf_counter()
    gpu = m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision=args.precision,
                                            device=local_rank)
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
    clk = clocks.stop()
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
    for _ in range(args.warmup):
        gpu.run(F_host, sig_host, update_coords=False)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gpu.run(F_host, sig_host, update_coords=False)
    barrier()
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = world * fiber_steps * args.steps / e2e_s
    ok_frac = float(np.mean(gpu.last_status["status"] == 0))

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
                   "parallelism": f"rve-sharded x{world}", "setup_s": round(setup_s, 2)},
        "rve_solves_per_s": world * R * args.steps / (t_ms * 1e-3),
        "e2e": {"value": e2e, "unit": "fiber-steps/s", "h2d_bytes_per_step": int(F_host.nbytes),
                "d2h_bytes_per_step": int(sig_host.nbytes + 16 * R)},
        "gpu_launches": int(launches_per_step * args.steps),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": f"{peak_kind} hbm_gbs",
                     "kernel": "relax_f64_kernel" if args.precision == "f64" else "relax_mixed",
                     "kernel_ms": relax_ms},
        "converged_or_completed_frac": ok_frac,
    }
    if clk:
        line["clocks"] = clk
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, args.cpu_sample_rves, os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    gpu.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
