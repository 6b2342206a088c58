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
