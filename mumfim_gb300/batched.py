"""Host-side mirror of the reference's batched microscale analysis.

``BatchedFiberRVEAnalysisExplicit`` keeps the method set of
``mumfim::BatchedRVEAnalysis`` (src/mumfim/microscale/BatchedRVEAnalysis.h:10-53)
and the constructor arguments of
``mumfim::BatchedFiberRVEAnalysisExplicit``
(src/mumfim/microscale/BatchedFiberRVEAnalysisExplicit.h:80-83): a list of
fiber networks and one solution strategy per network. Every call goes through
the C ABI of libmumfim_gpu.so (include/mumfim_gpu.h); nothing is computed in
Python and there is no CPU fallback: without the library or a GB300 the
constructor raises.

Arrays follow the reference's DualView shapes on the host: F is (n_rve, 3, 3)
(or (1, 3, 3) to broadcast), sigma (n_rve, 6) in Voigt order
[xx, yy, zz, yz, xz, xy], C (n_rve, 6, 6), omega (n_rve, 3, 3).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Sequence

import numpy as np

from . import _abi
from ._abi import (MFG_E_NOT_CONVERGED, MFG_E_NONFINITE, MFG_OK, MFG_PREC_F64, MFG_PREC_MIXED,
                   NetworkArray, RVE_STATUS_DTYPE, STATUS_NAMES, dptr)

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libmumfim_gpu.so")
# MFG_NOALLOC_SCRATCH_BYTES: size of the fixed device array the no-allocation
# solve takes its scratch from
NOALLOC_SCRATCH_BYTES = 16 << 20

_lib = None


class MumfimGpuError(RuntimeError):
    """A C-ABI call returned an error status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load_library(path: str | None = None):
    """Loads libmumfim_gpu.so (built by mumfim_gb300.build). Raises if it is
    missing: the package has no other implementation."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} is missing; build it with `python -m mumfim_gb300.build`")
    L = C.CDLL(p)
    vp, i32, dp = C.c_void_p, C.c_int32, C.POINTER(C.c_double)
    L.mfg_abi_version.restype = i32
    L.mfg_status_string.restype = C.c_char_p
    L.mfg_status_string.argtypes = [i32]
    L.mfg_last_error.restype = C.c_char_p
    L.mfg_batch_create.restype = i32
    L.mfg_batch_create.argtypes = [C.POINTER(_abi.mfg_network), C.POINTER(_abi.mfg_strategy), i32,
                                   C.POINTER(_abi.mfg_options), C.POINTER(vp)]
    L.mfg_batch_destroy.restype = i32
    L.mfg_batch_destroy.argtypes = [vp]
    for n in ("mfg_batch_n_nodes", "mfg_batch_n_fibers"):
        getattr(L, n).restype = i32
        getattr(L, n).argtypes = [vp, i32]
    L.mfg_batch_size.restype = i32
    L.mfg_batch_size.argtypes = [vp]
    L.mfg_batch_run.restype = i32
    L.mfg_batch_run.argtypes = [vp, dp, i32, dp, i32, vp]
    L.mfg_batch_run_device.restype = i32
    L.mfg_batch_run_device.argtypes = [vp, vp, i32, vp, i32, vp, vp]
    L.mfg_batch_run_device_noalloc.restype = i32
    L.mfg_batch_run_device_noalloc.argtypes = [vp, vp, i32, vp, i32, vp, vp]
    L.mfg_batch_material_stiffness.restype = i32
    L.mfg_batch_material_stiffness.argtypes = [vp, dp]
    L.mfg_batch_orientation_3d.restype = i32
    L.mfg_batch_orientation_3d.argtypes = [vp, dp]
    L.mfg_batch_orientation_2d.restype = i32
    L.mfg_batch_orientation_2d.argtypes = [vp, dp, dp]
    for n in ("mfg_batch_get_displacements", "mfg_batch_get_coordinates"):
        getattr(L, n).restype = i32
        getattr(L, n).argtypes = [vp, i32, dp]
    L.mfg_batch_get_current_stress.restype = i32
    L.mfg_batch_get_current_stress.argtypes = [vp, dp]
    L.mfg_batch_state_bytes.restype = C.c_size_t
    L.mfg_batch_state_bytes.argtypes = [vp, i32]
    for n in ("mfg_batch_export_state", "mfg_batch_import_state"):
        getattr(L, n).restype = i32
        getattr(L, n).argtypes = [vp, i32, vp, C.c_size_t]
    L.mfg_batch_last_timing.restype = i32
    L.mfg_batch_last_timing.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.mfg_batch_last_launches.restype = i32
    L.mfg_batch_last_launches.argtypes = [vp]
    L.mfg_set_metrics_log.restype = i32
    L.mfg_set_metrics_log.argtypes = [C.c_char_p]
    _lib = L
    return L


def set_metrics_log(path: str | None) -> None:
    """mfg_set_metrics_log(): append one JSON line per C-ABI call (create,
    run, stiffness, server poll) to `path`; None turns it off."""
    load_library().mfg_set_metrics_log(path.encode() if path else None)


def _check(status: int, allow=(MFG_OK,)):
    if status not in allow:
        msg = load_library().mfg_last_error().decode(errors="replace")
        raise MumfimGpuError(status, msg)
    return status


class BatchedFiberRVEAnalysisExplicit:
    """GPU batched explicit fiber-network RVE analysis.

    networks    sequence of network_io.FiberNetwork (reaction 0 drives the solve)
    strategies  one strategy.SolutionStrategy per network
    precision   "f64" (plain kernel, bit-identical to a serial CPU run) or "mixed"
    max_cluster_ctas  mixed precision: largest thread-block cluster an RVE may be
                split over (1, 2, 4 or 8; 0 = 8); results do not depend on it
    serving_layout  mixed precision: RVEs that need a cluster get clusters of 4
                (never 2), the layout the serving kernel uses; same results
    stiffness   "auto", "sequential" or "concurrent": how computeMaterialStiffness
                runs its six perturbed solves (mfg_stiffness_solves in
                include/mumfim_gpu.h)
    small_rve_solve  mixed precision: "auto" (= "node"), "node" or "fiber": the solve of
                RVEs whose node state fits one CTA (mfg_small_rve_solve); same results
    small_rves_per_cta  mixed precision, "fiber" only: 1 or 2 small RVEs per CTA (0 = 2)
    """

    def __init__(self, networks: Sequence, strategies: Sequence, precision: str = "f64",
                 device: int = 0, max_cluster_ctas: int = 0, serving_layout: bool = False,
                 stiffness: str = "auto", small_rves_per_cta: int = 0,
                 small_rve_solve: str = "auto"):
        L = load_library()
        if len(networks) != len(strategies):
            raise ValueError("There must be a solution strategy for each fiber network!")
        self._arr = NetworkArray(networks, strategies)
        opts = _abi.mfg_options()
        opts.precision = {"f64": MFG_PREC_F64, "mixed": MFG_PREC_MIXED}[precision]
        opts.device = device
        opts.max_cluster_ctas = max_cluster_ctas
        opts.cluster_layout = 1 if serving_layout else 0
        opts.stiffness = _abi.MFG_STIFFNESS[stiffness]
        opts.small_rves_per_cta = small_rves_per_cta
        opts.small_rve_solve = _abi.MFG_SMALL_RVE_SOLVE[small_rve_solve]
        h = C.c_void_p()
        _check(L.mfg_batch_create(self._arr.nets, self._arr.strats, len(networks), C.byref(opts),
                                  C.byref(h)))
        self._h = h
        self.num_rves = len(networks)
        self.precision = precision
        self.last_status = np.zeros(self.num_rves, dtype=RVE_STATUS_DTYPE)

    # -- lifecycle ------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            load_library().mfg_batch_destroy(self._h)
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

    @property
    def handle(self):
        return self._h

    def n_nodes(self, rve: int) -> int:
        return load_library().mfg_batch_n_nodes(self._h, rve)

    def n_fibers(self, rve: int) -> int:
        return load_library().mfg_batch_n_fibers(self._h, rve)

    # -- BatchedRVEAnalysis methods -------------------------------------------
    def run(self, dfmGrds, sigma=None, update_coords: bool = True) -> bool:
        """BatchedRVEAnalysis::run (BatchedRVEAnalysis.h:29-31). Fills sigma
        (n_rve x 6) in place when given and returns True when every RVE
        converged; per-RVE outcomes are in ``last_status``. Non-convergence
        and non-finite results are reported, not raised; bad arguments and
        CUDA failures raise MumfimGpuError."""
        F = np.ascontiguousarray(dfmGrds, dtype=np.float64).reshape(-1, 9)
        out = np.zeros((self.num_rves, 6)) if sigma is None else sigma
        buf = out if (out.dtype == np.float64 and out.flags["C_CONTIGUOUS"]) else \
            np.zeros((self.num_rves, 6))
        st = np.zeros(self.num_rves, dtype=RVE_STATUS_DTYPE)
        rc = load_library().mfg_batch_run(self._h, dptr(F), F.shape[0], dptr(buf),
                                          int(bool(update_coords)),
                                          st.ctypes.data_as(C.c_void_p))
        _check(rc, allow=(MFG_OK, MFG_E_NOT_CONVERGED, MFG_E_NONFINITE))
        if buf is not out:
            out[...] = buf
        self.last_status = st
        self.last_sigma = out
        return rc == MFG_OK

    def computeMaterialStiffness(self, C_out=None):
        """BatchedRVEAnalysis::computeMaterialStiffness (BatchedRVEAnalysis.h:36-37)."""
        Cm = np.zeros((self.num_rves, 6, 6))
        rc = load_library().mfg_batch_material_stiffness(self._h, dptr(Cm))
        _check(rc, allow=(MFG_OK, MFG_E_NOT_CONVERGED, MFG_E_NONFINITE))
        if C_out is not None:
            C_out[...] = Cm
            return C_out
        return Cm

    def compute3DOrientationTensor(self, omega=None):
        """BatchedRVEAnalysis::compute3DOrientationTensor (BatchedRVEAnalysis.h:38-43)."""
        om = np.zeros((self.num_rves, 3, 3))
        _check(load_library().mfg_batch_orientation_3d(self._h, dptr(om)))
        if omega is not None:
            omega[...] = om
            return omega
        return om

    def compute2DOrientationTensor(self, normal, omega=None):
        """BatchedRVEAnalysis::compute2DOrientationTensor (BatchedRVEAnalysis.h:44-50)."""
        nv = np.ascontiguousarray(np.broadcast_to(np.asarray(normal, dtype=np.float64).reshape(-1, 3),
                                                  (self.num_rves, 3)))
        om = np.zeros((self.num_rves, 3, 3))
        _check(load_library().mfg_batch_orientation_2d(self._h, dptr(nv), dptr(om)))
        if omega is not None:
            omega[...] = om
            return omega
        return om

    # -- state ----------------------------------------------------------------
    def displacements(self, rve: int) -> np.ndarray:
        u = np.zeros((self.n_nodes(rve), 3))
        _check(load_library().mfg_batch_get_displacements(self._h, rve, dptr(u)))
        return u

    def coordinates(self, rve: int) -> np.ndarray:
        x = np.zeros((self.n_nodes(rve), 3))
        _check(load_library().mfg_batch_get_coordinates(self._h, rve, dptr(x)))
        return x

    def current_stress(self) -> np.ndarray:
        s = np.zeros((self.num_rves, 6))
        _check(load_library().mfg_batch_get_current_stress(self._h, dptr(s)))
        return s

    def export_state(self, rve: int) -> bytes:
        L = load_library()
        n = L.mfg_batch_state_bytes(self._h, rve)
        buf = C.create_string_buffer(n)
        _check(L.mfg_batch_export_state(self._h, rve, buf, n))
        return buf.raw

    def import_state(self, rve: int, state: bytes):
        L = load_library()
        buf = C.create_string_buffer(state, len(state))
        _check(L.mfg_batch_import_state(self._h, rve, buf, len(state)))

    # -- device-resident path and timing ----------------------------------------
    def run_device(self, F_ptr: int, n_F: int, sigma_ptr: int, update_coords: bool = True,
                   status_ptr: int = 0, stream: int = 0):
        """Enqueues a solve on device-resident F / sigma (raw device pointers,
        e.g. torch tensor.data_ptr()) on `stream` without synchronising."""
        _check(load_library().mfg_batch_run_device(self._h, C.c_void_p(F_ptr), n_F,
                                                   C.c_void_p(sigma_ptr), int(bool(update_coords)),
                                                   C.c_void_p(status_ptr or None),
                                                   C.c_void_p(stream or None)))

    def run_device_noalloc(self, F_ptr: int, n_F: int, sigma_ptr: int, update_coords: bool = True,
                           status_ptr: int = 0, stream: int = 0):
        """mfg_batch_run_device_noalloc(): the FP64 solve of run_device() for
        callers that must not allocate device memory while solving; the
        kernel's scratch comes from the library's fixed device array (see
        include/mumfim_gpu.h for the size limit and the sharing rules)."""
        _check(load_library().mfg_batch_run_device_noalloc(
            self._h, C.c_void_p(F_ptr), n_F, C.c_void_p(sigma_ptr), int(bool(update_coords)),
            C.c_void_p(status_ptr or None), C.c_void_p(stream or None)))

    def last_timing(self):
        """(relaxation kernel ms, whole run ms) of the last run, CUDA events."""
        a, b = C.c_float(), C.c_float()
        _check(load_library().mfg_batch_last_timing(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def last_launches(self) -> int:
        return load_library().mfg_batch_last_launches(self._h)
