"""Continuous-batching RVE server (mfg_server_* in include/mumfim_gpu.h).

Replaces the blocking per-iteration batch of the multiscale service loop
(src/mumfim/microscale/MultiscaleRVEAnalysis.cc:197-305): integration points
submit deformation-gradient increments as they arrive and collect stresses as
they complete, while every RVE's state stays on the GPU between requests.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _abi
from ._abi import MFG_OK, MFG_PREC_F64, MFG_PREC_MIXED, NetworkArray, SERVER_RESULT_DTYPE, dptr
from .batched import MumfimGpuError, _check, load_library
from .strategy import SolutionStrategy

MFG_E_TIMEOUT = 5


def _lib():
    L = load_library()
    if not getattr(L, "_server_ready", False):
        vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
        L.mfg_server_create.restype = i32
        L.mfg_server_create.argtypes = [C.POINTER(_abi.mfg_network), C.POINTER(_abi.mfg_strategy),
                                        i32, C.POINTER(_abi.mfg_server_options), C.POINTER(vp)]
        L.mfg_server_submit.restype = i32
        L.mfg_server_submit.argtypes = [vp, i32, C.POINTER(C.c_double), i32, C.POINTER(i64)]
        L.mfg_server_submit_ex.restype = i32
        L.mfg_server_submit_ex.argtypes = [vp, i32, C.POINTER(C.c_double), i32, i32,
                                           C.POINTER(i64)]
        L.mfg_server_poll.restype = i32
        L.mfg_server_poll.argtypes = [vp, vp, i32, C.POINTER(i32), i32]
        L.mfg_server_outstanding.restype = i64
        L.mfg_server_outstanding.argtypes = [vp]
        L.mfg_server_launches.restype = i64
        L.mfg_server_launches.argtypes = [vp]
        L.mfg_server_batch.restype = vp
        L.mfg_server_batch.argtypes = [vp]
        L.mfg_server_destroy.restype = i32
        L.mfg_server_destroy.argtypes = [vp]
        L.mfg_device_bytes_estimate.restype = C.c_double
        L.mfg_device_bytes_estimate.argtypes = [C.POINTER(_abi.mfg_network), i32, i32]
        L._server_ready = True
    return L


class RVEServer:
    """Device-resident RVE pool served by a persistent kernel.

    submit(rve, F, update_coords) -> ticket   (non-blocking)
    poll(max, timeout_ms)         -> structured array of completed results
    """

    def __init__(self, networks: Sequence, strategies: Sequence, precision: str = "mixed",
                 device: int = 0, capacity: int = 0, idle_timeout_us: int = 0,
                 hbm_budget_bytes: float = 0.0, max_wait_ms: int = 0):
        L = _lib()
        self._arr = NetworkArray(networks, strategies)
        o = _abi.mfg_server_options()
        o.precision = {"f64": MFG_PREC_F64, "mixed": MFG_PREC_MIXED}[precision]
        o.device = device
        o.capacity = capacity
        o.idle_timeout_us = idle_timeout_us
        o.hbm_budget_bytes = hbm_budget_bytes
        o.max_wait_ms = max_wait_ms
        h = C.c_void_p()
        _check(L.mfg_server_create(self._arr.nets, self._arr.strats, len(networks), C.byref(o),
                                   C.byref(h)))
        self._h = h
        self.num_rves = len(networks)

    def close(self):
        if getattr(self, "_h", None):
            _lib().mfg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, rve: int, F, update_coords: bool = True, stiffness: bool = False) -> int:
        """Queues one solve; with stiffness=True the result also carries the
        RVE's material stiffness (field C, (6, 6), as computeMaterialStiffness
        returns it), from six perturbed solves run right after this one."""
        Fv = np.ascontiguousarray(np.asarray(F, dtype=np.float64).reshape(9))
        t = C.c_int64()
        _check(_lib().mfg_server_submit_ex(self._h, int(rve), dptr(Fv), int(bool(update_coords)),
                                           int(bool(stiffness)), C.byref(t)))
        return t.value

    def poll(self, max_results: int = 4096, timeout_ms: int = 1000) -> np.ndarray:
        """Completed results (possibly none). A wait that runs out is not an
        error here; poll_status() returns the C status as well."""
        return self.poll_status(max_results, timeout_ms)[0]

    def poll_status(self, max_results: int = 4096, timeout_ms: int = 1000):
        """(results, mfg_server_poll status): MFG_OK, or MFG_E_TIMEOUT when
        work is outstanding and nothing completed within timeout_ms."""
        out = np.zeros(max_results, dtype=SERVER_RESULT_DTYPE)
        n = C.c_int32()
        rc = _lib().mfg_server_poll(self._h, out.ctypes.data_as(C.c_void_p), max_results,
                                    C.byref(n), int(timeout_ms))
        _check(rc, allow=(MFG_OK, MFG_E_TIMEOUT))
        return out[:n.value], rc

    def drain(self, timeout_s: float = 600.0) -> np.ndarray:
        """Polls until nothing is outstanding; returns every result."""
        import time
        parts = []
        t_end = time.monotonic() + timeout_s
        while self.outstanding() > 0:
            if time.monotonic() > t_end:
                raise MumfimGpuError(MFG_E_TIMEOUT, "drain timed out")
            parts.append(self.poll(timeout_ms=200))
        return np.concatenate(parts) if parts else np.zeros(0, dtype=SERVER_RESULT_DTYPE)

    def outstanding(self) -> int:
        return int(_lib().mfg_server_outstanding(self._h))

    def launches(self) -> int:
        return int(_lib().mfg_server_launches(self._h))

    def export_state(self, rve: int) -> bytes:
        """One RVE's persistent state (mfg_batch_export_state on the server's
        batch); valid while no request is outstanding."""
        L = _lib()
        b = L.mfg_server_batch(self._h)
        n = L.mfg_batch_state_bytes(b, int(rve))
        buf = C.create_string_buffer(n)
        _check(L.mfg_batch_export_state(b, int(rve), buf, n))
        return buf.raw

    def import_state(self, rve: int, state: bytes) -> None:
        L = _lib()
        buf = C.create_string_buffer(state, len(state))
        _check(L.mfg_batch_import_state(L.mfg_server_batch(self._h), int(rve), buf, len(state)))


def device_bytes_estimate(networks: Sequence, precision: str = "mixed") -> float:
    """mfg_device_bytes_estimate(): device memory of a batch of `networks`."""
    arr = NetworkArray(networks, [SolutionStrategy()] * len(networks))
    prec = {"f64": MFG_PREC_F64, "mixed": MFG_PREC_MIXED}[precision]
    return float(_lib().mfg_device_bytes_estimate(arr.nets, len(networks), prec))


class PagedRVEServer:
    """Continuous-batching service over more RVEs than a device-memory budget
    holds: admission per request, eviction of idle RVEs to host memory.

    The RVEs are grouped into pages of `page_size` consecutive ids. A page
    is made resident -- its own RVEServer, so its RVEs' state lives on the
    device -- when a request for one of its RVEs arrives. If the estimated
    device memory of the resident pages and the new one
    (mfg_device_bytes_estimate) would exceed `hbm_budget_bytes`, the least
    recently used pages without a request in flight are evicted first: every
    RVE's persistent state (displacements, coordinates, volume, last stress)
    is exported to host memory and the page's device memory is freed. A
    re-admitted page gets its saved states back. A request whose page cannot
    be admitted yet (the budget is held by pages with requests in flight)
    waits on the host, and requests for one RVE keep their order. The solve
    depends only on the network, the state and the request, so every result
    is bit-identical to that of one server holding all RVEs.

    Each resident page runs its own persistent kernel; the kernels share the
    GPU, a page's kernel leaving after `idle_timeout_us` without work, so
    large pages (few of them resident) keep the GPU busiest.
    """

    def __init__(self, networks: Sequence, strategies: Sequence, hbm_budget_bytes: float,
                 page_size: int = 1024, precision: str = "mixed", device: int = 0,
                 idle_timeout_us: int = 2000):
        from collections import OrderedDict, deque
        if page_size < 1:
            raise ValueError("page_size must be >= 1")
        self.networks, self.strategies = list(networks), list(strategies)
        self.n = len(self.networks)
        self.precision, self.device, self.idle_us = precision, device, idle_timeout_us
        self.pages = [list(range(i, min(i + page_size, self.n)))
                      for i in range(0, self.n, page_size)]
        self.page_bytes = [device_bytes_estimate([self.networks[r] for r in pg], precision)
                           for pg in self.pages]
        self.budget = float(hbm_budget_bytes)
        if max(self.page_bytes) > self.budget:
            raise MumfimGpuError(8, f"admission refused: a page needs {max(self.page_bytes):.3g} "
                                    f"bytes, the budget is {self.budget:.3g}")
        self.resident = OrderedDict()  # page -> RVEServer, least recently used first
        self.in_flight = [0] * len(self.pages)
        self.saved = {}  # rve -> exported state of an evicted page
        self.waiting = deque()  # (ticket, rve, F, update, stiffness)
        self.tickets = {}  # (page, page-local ticket) -> ticket
        self.next_ticket = 0
        self.evictions = 0
        self.admissions = 0

    def _page(self, rve):
        return rve // len(self.pages[0])

    def _admit(self, pg) -> bool:
        if pg in self.resident:
            self.resident.move_to_end(pg)
            return True
        used = sum(self.page_bytes[p] for p in self.resident)
        for p in list(self.resident):  # evict idle pages, least recently used first
            if used + self.page_bytes[pg] <= self.budget:
                break
            if self.in_flight[p] == 0:
                sv = self.resident.pop(p)
                for i, r in enumerate(self.pages[p]):
                    self.saved[r] = sv.export_state(i)
                sv.close()
                used -= self.page_bytes[p]
                self.evictions += 1
        if used + self.page_bytes[pg] > self.budget:
            return False
        ids = self.pages[pg]
        sv = RVEServer([self.networks[r] for r in ids], [self.strategies[r] for r in ids],
                       precision=self.precision, device=self.device,
                       idle_timeout_us=self.idle_us, hbm_budget_bytes=self.page_bytes[pg] * 1.01)
        for i, r in enumerate(ids):
            if r in self.saved:
                sv.import_state(i, self.saved.pop(r))
        self.resident[pg] = sv
        self.admissions += 1
        return True

    def _pump(self):
        blocked = set()  # pages with an earlier request still waiting: keep per-RVE order
        keep = []
        for req in self.waiting:
            t, rve, F, upd, stiff = req
            pg = self._page(rve)
            if pg in blocked or not self._admit(pg):
                blocked.add(pg)
                keep.append(req)
                continue
            lt = self.resident[pg].submit(rve - self.pages[pg][0], F, upd, stiff)
            self.tickets[(pg, lt)] = t
            self.in_flight[pg] += 1
        self.waiting.clear()
        self.waiting.extend(keep)

    def submit(self, rve: int, F, update_coords: bool = True, stiffness: bool = False) -> int:
        if not 0 <= rve < self.n:
            raise MumfimGpuError(1, f"rve {rve} out of range")
        t = self.next_ticket
        self.next_ticket += 1
        self.waiting.append((t, int(rve), np.asarray(F, dtype=np.float64).reshape(3, 3).copy(),
                             bool(update_coords), bool(stiffness)))
        self._pump()
        return t

    def outstanding(self) -> int:
        return len(self.waiting) + sum(self.in_flight)

    def poll(self, max_results: int = 4096, timeout_ms: int = 1000) -> np.ndarray:
        import time
        t_end = time.monotonic() + 1e-3 * timeout_ms
        while True:
            parts = []
            for pg, sv in list(self.resident.items()):
                if self.in_flight[pg] == 0:
                    continue
                res = sv.poll(max_results, timeout_ms=0)
                if len(res):
                    res = res.copy()
                    for k in range(len(res)):
                        res["ticket"][k] = self.tickets.pop((pg, int(res["ticket"][k])))
                    res["rve"] += self.pages[pg][0]
                    self.in_flight[pg] -= len(res)
                    parts.append(res)
            self._pump()
            if parts:
                return np.concatenate(parts)
            if self.outstanding() == 0 or time.monotonic() >= t_end:
                return np.zeros(0, dtype=SERVER_RESULT_DTYPE)
            time.sleep(5e-5)

    def drain(self, timeout_s: float = 600.0) -> np.ndarray:
        import time
        parts = []
        t_end = time.monotonic() + timeout_s
        while self.outstanding() > 0:
            if time.monotonic() > t_end:
                raise MumfimGpuError(MFG_E_TIMEOUT, "drain timed out")
            parts.append(self.poll(timeout_ms=200))
        return np.concatenate(parts) if parts else np.zeros(0, dtype=SERVER_RESULT_DTYPE)

    def close(self):
        for sv in self.resident.values():
            sv.close()
        self.resident.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
