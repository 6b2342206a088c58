"""ctypes mirror of the structs in include/mumfim_gpu.h."""
from __future__ import annotations

import ctypes as C

import numpy as np

MFG_OK = 0
MFG_E_INVALID = 1
MFG_E_OOM = 2
MFG_E_NOT_CONVERGED = 3
MFG_E_NONFINITE = 4
MFG_E_TIMEOUT = 5
MFG_E_CUDA = 6
MFG_E_NO_DEVICE = 7
MFG_E_BUSY = 8

STATUS_NAMES = {
    MFG_OK: "MFG_OK", MFG_E_INVALID: "MFG_E_INVALID", MFG_E_OOM: "MFG_E_OOM",
    MFG_E_NOT_CONVERGED: "MFG_E_NOT_CONVERGED", MFG_E_NONFINITE: "MFG_E_NONFINITE",
    MFG_E_TIMEOUT: "MFG_E_TIMEOUT", MFG_E_CUDA: "MFG_E_CUDA",
    MFG_E_NO_DEVICE: "MFG_E_NO_DEVICE", MFG_E_BUSY: "MFG_E_BUSY",
}

MFG_LAW_LINEAR = 0
MFG_LAW_NONLINEAR = 1
MFG_MODE_RELAX = 0
MFG_MODE_RAMP = 1
MFG_PREC_F64 = 0
MFG_PREC_MIXED = 1
MFG_STIFFNESS = {"auto": 0, "sequential": 1, "concurrent": 2}
MFG_SMALL_RVE_SOLVE = {"auto": 0, "node": 1, "fiber": 2}


class mfg_reaction(C.Structure):
    _fields_ = [("law", C.c_int32), ("pad_", C.c_int32), ("radius", C.c_double),
                ("youngs_modulus", C.c_double), ("density", C.c_double), ("B", C.c_double),
                ("length_ratio_trns", C.c_double)]


class mfg_network(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("n_fibers", C.c_int32),
                ("coords", C.POINTER(C.c_double)), ("connectivity", C.POINTER(C.c_int32)),
                ("reaction", mfg_reaction), ("scale_factor", C.c_double)]


class mfg_strategy(C.Structure):
    _fields_ = [("visc_damp_coeff", C.c_double), ("crit_time_scale_factor", C.c_double),
                ("residual_tol", C.c_double), ("max_steps", C.c_int32), ("mode", C.c_int32)]


class mfg_options(C.Structure):
    _fields_ = [("precision", C.c_int32), ("device", C.c_int32),
                ("threads_per_rve", C.c_int32), ("max_cluster_ctas", C.c_int32),
                ("cluster_layout", C.c_int32), ("stiffness", C.c_int32),
                ("small_rves_per_cta", C.c_int32), ("small_rve_solve", C.c_int32)]


class mfg_rve_status(C.Structure):
    _fields_ = [("status", C.c_int32), ("steps", C.c_int32), ("residual", C.c_double)]


RVE_STATUS_DTYPE = np.dtype([("status", np.int32), ("steps", np.int32), ("residual", np.float64)])


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class NetworkArray:
    """Keeps numpy buffers alive for an array of mfg_network structs."""

    def __init__(self, networks, strategies):
        n = len(networks)
        if n != len(strategies):
            raise ValueError("There must be a solution strategy for each fiber network!")
        self._keep = []
        self.nets = (mfg_network * n)()
        self.strats = (mfg_strategy * n)()
        for i, (net, s) in enumerate(zip(networks, strategies)):
            coords = np.ascontiguousarray(net.coords, dtype=np.float64)
            conn = np.ascontiguousarray(net.connectivity, dtype=np.int32)
            self._keep += [coords, conn]
            r = net.reactions[0]
            self.nets[i] = mfg_network(
                int(coords.shape[0]), int(conn.shape[0]), dptr(coords), iptr(conn),
                mfg_reaction(int(r.law), 0, float(r.radius), float(r.youngs_modulus),
                             float(r.density), float(r.B), float(r.length_ratio_trns)),
                float(net.scale_factor))
            self.strats[i] = mfg_strategy(float(s.visc_damp_coeff), float(s.crit_time_scale_factor),
                                          float(s.residual_tol), int(s.max_steps), int(s.mode))
        self.n = n


class mfg_server_options(C.Structure):
    _fields_ = [("precision", C.c_int32), ("device", C.c_int32), ("capacity", C.c_int32),
                ("idle_timeout_us", C.c_int32), ("hbm_budget_bytes", C.c_double),
                ("max_wait_ms", C.c_int32), ("reserved", C.c_int32 * 3)]


SERVER_RESULT_DTYPE = np.dtype([("ticket", np.int64), ("rve", np.int32), ("status", np.int32),
                                ("steps", np.int32), ("stiffness_status", np.int32),
                                ("residual", np.float64), ("sigma", np.float64, (6,)),
                                ("latency_s", np.float64), ("device_s", np.float64),
                                ("t_claim_ns", np.int64), ("t_done_ns", np.int64),
                                ("C", np.float64, (6, 6))])
