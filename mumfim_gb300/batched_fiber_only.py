"""Standalone batched fiber-network run, the counterpart of the reference's
``batched_fiber_only job.yaml num_rves`` driver (src/batched_fiber_only.cc):
the first case of the job file gives the network, the deformation gradient
and the damping; the network is replicated num_rves times; the driver prints
RVE 0's 3-D orientation tensor and its 2-D one about the x axis, runs the
batch, prints RVE 0's stress and material stiffness, and the times taken.

    python -m mumfim_gb300.batched_fiber_only job.yaml num_rves [--precision f64|mixed]
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import BatchedFiberRVEAnalysisExplicit, load_network
from .jobfile import load_micro_cases, resolve_mesh


def _print_tensor(t) -> None:
    for i in range(3):
        print("".join(f"{t[i, j]:f} " for j in range(3)))
    print()


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m mumfim_gb300.batched_fiber_only",
                                 description=__doc__.split("\n\n")[0])
    ap.add_argument("job", help="job file (fiber_only.yaml format)")
    ap.add_argument("num_rves", type=int)
    ap.add_argument("--precision", default="f64", choices=["f64", "mixed"])
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--json", default=None, help="also write RVE 0's results at full precision")
    args = ap.parse_args(argv)
    if args.num_rves < 1:
        ap.error("num_rves must be positive")
    cases = load_micro_cases(args.job)
    c = cases[0]
    print(f"{c.name}\n\t{c.mesh}\n\tF=[" + "; ".join(
        " ".join(f"{c.F[3 * i + j]:g}" for j in range(3)) for i in range(3)) + "]")
    mesh = resolve_mesh(c, args.job)
    net = load_network(mesh, mesh + ".params")
    n = args.num_rves
    analysis = BatchedFiberRVEAnalysisExplicit([net] * n, [c.strategy()] * n,
                                               precision=args.precision, device=args.device)
    F = np.repeat(np.array(c.F, dtype=np.float64).reshape(1, 3, 3), n, 0)
    normal = np.repeat(np.array([[1.0, 0.0, 0.0]]), n, 0)
    t0 = time.perf_counter()
    o3 = analysis.compute3DOrientationTensor()
    _print_tensor(o3[0])
    o2 = analysis.compute2DOrientationTensor(normal)
    _print_tensor(o2[0])
    t1 = time.perf_counter()
    sigma = np.zeros((n, 6))
    analysis.run(F, sigma)
    s = sigma[0]
    S = np.array([[s[0], s[5], s[4]], [s[5], s[1], s[3]], [s[4], s[3], s[2]]])
    print()
    for i in range(3):
        print(" ".join(f"{S[i, j]:g}" for j in range(3)))
    C = analysis.computeMaterialStiffness()
    for i in range(6):
        print(" ".join(f"{C[0].reshape(6, 6)[i, j]:g}" for j in range(6)) + " ")
    print()
    t2 = time.perf_counter()
    print(f"Took: {t2 - t1:g} seconds.")
    print(f"Orientation Computation Took: {t1 - t0:g} seconds.")
    status = analysis.last_status
    if args.json:
        with open(args.json, "w") as fh:
            json.dump({"sigma": sigma[0].tolist(), "stiffness": np.asarray(C[0]).ravel().tolist(),
                       "orientation_3d": o3[0].ravel().tolist(),
                       "orientation_2d": o2[0].ravel().tolist(),
                       "status": int(status["status"][0]), "steps": int(status["steps"][0])}, fh)
    analysis.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
