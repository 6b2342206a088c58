"""Seeded synthetic workloads of the benchmark configurations.

There is no public dataset for this path; these generators build the fiber
networks, material parameters and deformation gradients the configurations
describe, reproducibly from (config id, RVE id):

  config 0  1 RVE, 1000 nodes, k = 4 nearest-neighbour fibers, linear law
            r = 1e-3, E = 1, rho = 1, damping 0.5, F = diag(1.1, 1, 1) ramped
            over 10,000 steps at 0.8 x the critical step
  config 1  1024 RVEs of 4500 nodes, k = 4, r ~ lognormal(ln 1e-3, 0.2),
            E ~ lognormal(0, 0.3), rho = 1, F = I + symmetric U(+-0.05),
            5,000 steps
  config 2  4096 RVEs, nodes log-uniform in [500, 20000], k in {3, 4, 5},
            parameters as config 1, F = I + general U(+-0.08), 5,000 steps
  config 3  2048 RVEs, nodes log-uniform in [2000, 8000], exponential-toe
            law with E ~ lognormal(0, 0.3), B ~ U[1, 10], transition ratio
            ~ U[1.02, 1.15], r = 1e-3, F = uniaxial U[1, 1.25] x simple shear
            U(+-0.15), 20,000 steps

Nodes within 0.02 of a face are snapped onto it (they are the fixed
boundary); draws within 1e-6 of an earlier node are redrawn. All random
numbers come from std::mt19937_64 streams in the C library, so the same
ids give the same networks on x86-64 and aarch64.
"""
from __future__ import annotations

import ctypes as C
import os
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from typing import List

import numpy as np

from ._abi import MFG_MODE_RAMP, dptr
from .network_io import LINEAR, NONLINEAR, FiberNetwork, Reaction
from .strategy import SolutionStrategy

SNAP = 0.02
MIN_SEP = 1e-6


_netgen = None
_netgen_path = None


def use_netgen_library(path: str) -> None:
    """Takes the network generator from the shared library at `path` (a
    build of netgen.cpp) instead of mumfim_gb300/_lib/libmumfim_netgen.so;
    call before the first network is generated."""
    global _netgen_path
    if _netgen is not None and path != _netgen_path:
        raise RuntimeError("the network generator is already loaded")
    _netgen_path = path


def _lib():
    global _netgen
    if _netgen is None:
        from .build import NETGEN_PATH
        p = _netgen_path or NETGEN_PATH
        if not os.path.exists(p):
            raise ImportError(f"{p} is missing; build it with `python -m mumfim_gb300.build`")
        L = C.CDLL(p)
        L.mfg_generate_knn_network.restype = C.c_int32
        L.mfg_generate_knn_network.argtypes = [C.c_int32, C.c_int32, C.c_uint64, C.c_double,
                                               C.c_double, C.POINTER(C.c_double),
                                               C.POINTER(C.c_int32), C.c_int32]
        for n in ("mfg_generate_uniform", "mfg_generate_normal"):
            getattr(L, n).restype = None
            getattr(L, n).argtypes = [C.c_uint64, C.c_int32, C.POINTER(C.c_double)]
        for n in ("mfg_portable_exp", "mfg_portable_log"):
            getattr(L, n).restype = C.c_double
            getattr(L, n).argtypes = [C.c_double]
        _netgen = L
    return _netgen


def knn_network(n_nodes: int, k: int, seed: int, snap: float = SNAP, min_sep: float = MIN_SEP):
    """(coords (n,3) float64, connectivity (E,2) int32) of one seeded network."""
    L = _lib()
    coords = np.zeros((n_nodes, 3))
    cap = n_nodes * k
    conn = np.zeros((cap, 2), dtype=np.int32)
    ne = L.mfg_generate_knn_network(n_nodes, k, seed, snap, min_sep, dptr(coords),
                                    conn.ctypes.data_as(C.POINTER(C.c_int32)), cap)
    if ne < 0:
        raise ValueError("network generation failed")
    return coords, np.ascontiguousarray(conn[:ne])


def uniform(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n)
    _lib().mfg_generate_uniform(seed, n, dptr(out))
    return out


def normal(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n)
    _lib().mfg_generate_normal(seed, n, dptr(out))
    return out


def pexp(x: float) -> float:
    return _lib().mfg_portable_exp(float(x))


def plog(x: float) -> float:
    return _lib().mfg_portable_log(float(x))


def geometry_seed(config: int, rve: int) -> int:
    return ((config & 0xFFFFFFFF) << 32) | (rve & 0xFFFFFFFF)


def param_seed(config: int, rve: int) -> int:
    return geometry_seed(config, rve) ^ 0x5DEECE66D2545F49


@dataclass
class Workload:
    name: str
    networks: List[FiberNetwork]
    strategies: List[SolutionStrategy]
    F: np.ndarray  # (n_rve, 3, 3)
    steps: int

    @property
    def n_rve(self) -> int:
        return len(self.networks)

    @property
    def total_fibers(self) -> int:
        return int(sum(n.n_fibers for n in self.networks))

    @property
    def total_nodes(self) -> int:
        return int(sum(n.n_nodes for n in self.networks))

    def subset(self, idx) -> "Workload":
        idx = list(idx)
        return Workload(self.name + f"[{len(idx)}]", [self.networks[i] for i in idx],
                        [self.strategies[i] for i in idx], self.F[idx], self.steps)


def _parallel(fn, n):
    with ThreadPoolExecutor(max_workers=16) as ex:
        return list(ex.map(fn, range(n)))


def config0(steps: int = 10_000) -> Workload:
    coords, conn = knn_network(1000, 4, geometry_seed(0, 0))
    net = FiberNetwork(coords, conn, [Reaction(LINEAR, 1e-3, 1.0, 1.0)])
    F = np.diag([1.10, 1.0, 1.0]).reshape(1, 3, 3)
    return Workload("config0", [net], [SolutionStrategy.ramp(steps, 0.5)], F, steps)


def _linear_params(config: int, rve: int):
    z = normal(param_seed(config, rve), 2)
    r = pexp(plog(1e-3) + 0.2 * z[0])
    E = pexp(0.0 + 0.3 * z[1])
    return Reaction(LINEAR, r, E, 1.0)


def config1(n_rve: int = 1024, n_nodes: int = 4500, steps: int = 5_000, first: int = 0) -> Workload:
    def one(i):
        r = first + i
        coords, conn = knn_network(n_nodes, 4, geometry_seed(1, r))
        u = uniform(param_seed(1, r) + 1, 6) * 0.1 - 0.05
        A = np.array([[u[0], u[3], u[4]], [u[3], u[1], u[5]], [u[4], u[5], u[2]]])
        return FiberNetwork(coords, conn, [_linear_params(1, r)]), np.eye(3) + A

    res = _parallel(one, n_rve)
    nets = [r[0] for r in res]
    F = np.stack([r[1] for r in res])
    return Workload("config1", nets, [SolutionStrategy.ramp(steps, 0.5) for _ in nets], F, steps)


def config2(n_rve: int = 4096, steps: int = 5_000, first: int = 0,
            n_min: int = 500, n_max: int = 20_000) -> Workload:
    def one(i):
        r = first + i
        u = uniform(param_seed(2, r) + 1, 11)
        n = int(round(pexp(plog(n_min) + u[0] * (plog(n_max) - plog(n_min)))))
        k = 3 + min(int(u[1] * 3), 2)
        coords, conn = knn_network(n, k, geometry_seed(2, r))
        A = (u[2:11] * 0.16 - 0.08).reshape(3, 3)
        return FiberNetwork(coords, conn, [_linear_params(2, r)]), np.eye(3) + A

    res = _parallel(one, n_rve)
    nets = [r[0] for r in res]
    F = np.stack([r[1] for r in res])
    return Workload("config2", nets, [SolutionStrategy.ramp(steps, 0.5) for _ in nets], F, steps)


def config3(n_rve: int = 2048, steps: int = 20_000, first: int = 0,
            n_min: int = 2000, n_max: int = 8000) -> Workload:
    def one(i):
        r = first + i
        u = uniform(param_seed(3, r) + 1, 5)
        z = normal(param_seed(3, r), 1)
        n = int(round(pexp(plog(n_min) + u[0] * (plog(n_max) - plog(n_min)))))
        coords, conn = knn_network(n, 4, geometry_seed(3, r))
        E = pexp(0.3 * z[0])
        B = 1.0 + 9.0 * u[1]
        lt = 1.02 + 0.13 * u[2]
        stretch = 1.0 + 0.25 * u[3]
        shear = u[4] * 0.3 - 0.15
        F = np.diag([stretch, 1.0, 1.0]) @ np.array([[1.0, shear, 0.0], [0.0, 1.0, 0.0],
                                                      [0.0, 0.0, 1.0]])
        return FiberNetwork(coords, conn, [Reaction(NONLINEAR, 1e-3, E, 1.0, B, lt)]), F

    res = _parallel(one, n_rve)
    nets = [r[0] for r in res]
    F = np.stack([r[1] for r in res])
    return Workload("config3", nets, [SolutionStrategy.ramp(steps, 0.5) for _ in nets], F, steps)


def config4(n_points: int = 20_000, steps: int = 500, first: int = 0,
            n_min: int = 500, n_max: int = 20_000) -> Workload:
    """Serving stream: one persistent RVE per integration point, nodes
    log-uniform in [500, 20000], linear or exponential-toe law 50/50 with the
    distributions of configs 2 and 3; each request relaxes `steps` RAMP
    steps. F holds the identity; increments come from config4_increment()."""
    def one(i):
        r = first + i
        u = uniform(param_seed(4, r) + 1, 8)
        n = int(round(pexp(plog(n_min) + u[0] * (plog(n_max) - plog(n_min)))))
        k = 3 + min(int(u[1] * 3), 2)
        coords, conn = knn_network(n, k, geometry_seed(4, r))
        if u[2] < 0.5:
            rc = _linear_params(4, r)
        else:
            z = normal(param_seed(4, r), 1)
            rc = Reaction(NONLINEAR, 1e-3, pexp(0.3 * z[0]), 1.0, 1.0 + 9.0 * u[3],
                          1.02 + 0.13 * u[4])
        return FiberNetwork(coords, conn, [rc])

    nets = _parallel(one, n_points)
    F = np.repeat(np.eye(3)[None], n_points, 0)
    return Workload("config4", nets, [SolutionStrategy.ramp(steps, 0.5) for _ in nets], F, steps)


def config4_increment(point: int, load_step: int, iteration: int) -> np.ndarray:
    """Deformation-gradient increment of one request: I + U(+-0.005) entries."""
    seed = param_seed(4, point) ^ (((load_step & 0xFFFF) << 16) | (iteration & 0xFFFF)) ^ 0xABCDEF
    return np.eye(3) + (uniform(seed, 9) * 0.01 - 0.005).reshape(3, 3)


def poisson_arrivals(seed: int, n: int, rate: float) -> np.ndarray:
    """Arrival offsets (s) of a Poisson stream of n requests at `rate` per s."""
    u = uniform(seed, n)
    gaps = np.array([-plog(1.0 - x) for x in u]) / rate
    return np.cumsum(gaps)
