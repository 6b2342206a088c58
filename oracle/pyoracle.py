"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the mumfim_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

from mumfim_gb300._abi import (NetworkArray, RVE_STATUS_DTYPE, dptr, mfg_network,
                               mfg_rve_status, mfg_strategy)

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
FAST_LIB_PATH = os.path.join(BUILD_DIR, "liboracle_fast.so")
NETGEN_PATH = os.path.join(BUILD_DIR, "libnetgen.so")

# Parity build: no contraction and no target-specific code, so x86-64 and
# aarch64 give the same bits as the FP64 GPU kernel.
PARITY_FLAGS = ["-O2", "-ffp-contract=off"]


def timing_flags() -> list:
    """Timing build of the same source for the CPU baseline: -O3, loop
    unrolling, contraction into FMAs allowed, and the GPU machine's host core
    named explicitly (Neoverse V2 on aarch64). Its results differ from the
    parity build's in the last bits only (test_oracle_golden checks 1e-9)."""
    flags = ["-O3", "-funroll-loops", "-ffp-contract=fast"]
    if platform.machine() in ("aarch64", "arm64"):
        flags.append("-mcpu=neoverse-v2")
    return flags


def _compile(out: str, flags: list, force: bool) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "mumfim_oracle.cpp")
    deps = [src, os.path.join(HERE, "mumfim_oracle.h"), __file__]
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(
            os.path.getmtime(d) for d in deps):
        return out
    cmd = ["g++", *flags, "-std=c++17", "-fPIC", "-shared", "-pthread",
           "-I" + os.path.join(REPO, "include"), "-I" + HERE, src, "-o", out + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


def build(force: bool = False) -> str:
    """Compiles the oracle's parity build, its timing build and a copy of the
    network generator for the CPU-only reference arm; returns the parity
    build's path."""
    _compile(FAST_LIB_PATH, timing_flags(), force)
    build_netgen(force)
    return _compile(LIB_PATH, PARITY_FLAGS, force)


def build_netgen(force: bool = False) -> str:
    """The synthetic-network generator compiled into oracle/_build, so that
    the CPU-only reference arm of the benchmark maps no library of the
    product."""
    from mumfim_gb300.build import build_netgen as _bn
    return _bn(NETGEN_PATH, force)


_libs = {}


def lib(timing: bool = False):
    """The parity build (default) or the timing build, loaded with ctypes."""
    key = "timing" if timing else "parity"
    if key not in _libs:
        build()
        L = C.CDLL(FAST_LIB_PATH if timing else LIB_PATH)
        L.orc_batch_create.restype = C.c_void_p
        L.orc_batch_create.argtypes = [C.POINTER(mfg_network), C.POINTER(mfg_strategy), C.c_int32]
        L.orc_batch_destroy.argtypes = [C.c_void_p]
        L.orc_batch_run.restype = C.c_int32
        L.orc_batch_run.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int32,
                                    C.POINTER(C.c_double), C.c_int32, C.c_void_p, C.c_int32]
        L.orc_batch_material_stiffness.restype = C.c_int32
        L.orc_batch_material_stiffness.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int32]
        for name in ("orc_batch_orientation_3d",):
            getattr(L, name).restype = C.c_int32
            getattr(L, name).argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_batch_orientation_2d.restype = C.c_int32
        L.orc_batch_orientation_2d.argtypes = [C.c_void_p, C.POINTER(C.c_double),
                                               C.POINTER(C.c_double)]
        for name in ("orc_batch_get_displacements", "orc_batch_get_coordinates"):
            getattr(L, name).restype = C.c_int32
            getattr(L, name).argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]
        L.orc_batch_get_current_stress.restype = C.c_int32
        L.orc_batch_get_current_stress.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_reorder_permutation.argtypes = [C.c_int32, C.POINTER(C.c_int32), C.c_int32,
                                              C.POINTER(C.c_int32)]
        L.orc_boundary_nodes.restype = C.c_int32
        L.orc_boundary_nodes.argtypes = [C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int32)]
        L.orc_scale_conversion.restype = C.c_double
        L.orc_scale_conversion.argtypes = [C.c_int32, C.POINTER(C.c_double), C.c_int32,
                                           C.POINTER(C.c_int32), C.c_double, C.c_double]
        L.orc_nodal_mass.argtypes = [C.c_int32, C.POINTER(C.c_double), C.c_int32,
                                     C.POINTER(C.c_int32), C.c_double, C.c_double,
                                     C.POINTER(C.c_double)]
        _libs[key] = L
    return _libs[key]


class OracleBatch:
    """CPU restatement of BatchedFiberRVEAnalysisExplicit with the same
    arguments as mumfim_gb300.BatchedFiberRVEAnalysisExplicit."""

    def __init__(self, networks, strategies, timing: bool = False):
        """timing=True uses the optimised timing build (CPU baseline) instead
        of the bit-stable parity build."""
        self._L = lib(timing)
        self._arr = NetworkArray(networks, strategies)
        self.n_rve = len(networks)
        self.n_nodes = [n.n_nodes for n in networks]
        self._h = self._L.orc_batch_create(self._arr.nets, self._arr.strats, self.n_rve)
        if not self._h:
            raise ValueError("oracle rejected the networks")

    def close(self):
        if self._h:
            self._L.orc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def run(self, F, update_coords=True, n_threads=1):
        F = np.ascontiguousarray(F, dtype=np.float64).reshape(-1, 9)
        sigma = np.zeros((self.n_rve, 6))
        st = np.zeros(self.n_rve, dtype=RVE_STATUS_DTYPE)
        rc = self._L.orc_batch_run(self._h, dptr(F), F.shape[0], dptr(sigma), int(update_coords),
                                 st.ctypes.data_as(C.c_void_p), n_threads)
        return rc, sigma, st

    def material_stiffness(self, n_threads=1):
        Cm = np.zeros((self.n_rve, 6, 6))
        rc = self._L.orc_batch_material_stiffness(self._h, dptr(Cm), n_threads)
        return rc, Cm

    def orientation_3d(self):
        om = np.zeros((self.n_rve, 3, 3))
        self._L.orc_batch_orientation_3d(self._h, dptr(om))
        return om

    def orientation_2d(self, normal):
        normal = np.ascontiguousarray(normal, dtype=np.float64).reshape(self.n_rve, 3)
        om = np.zeros((self.n_rve, 3, 3))
        self._L.orc_batch_orientation_2d(self._h, dptr(normal), dptr(om))
        return om

    def displacements(self, rve):
        u = np.zeros((self.n_nodes[rve], 3))
        self._L.orc_batch_get_displacements(self._h, rve, dptr(u))
        return u

    def coordinates(self, rve):
        x = np.zeros((self.n_nodes[rve], 3))
        self._L.orc_batch_get_coordinates(self._h, rve, dptr(x))
        return x

    def current_stress(self):
        s = np.zeros((self.n_rve, 6))
        self._L.orc_batch_get_current_stress(self._h, dptr(s))
        return s


def reorder_permutation(n_vert, fixed):
    fixed = np.ascontiguousarray(fixed, dtype=np.int32)
    perm = np.zeros(n_vert, dtype=np.int32)
    lib().orc_reorder_permutation(n_vert, fixed.ctypes.data_as(C.POINTER(C.c_int32)),
                                  fixed.shape[0], perm.ctypes.data_as(C.POINTER(C.c_int32)))
    return perm


def boundary_nodes(coords):
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    out = np.zeros(coords.shape[0], dtype=np.int32)
    nb = lib().orc_boundary_nodes(coords.shape[0], dptr(coords),
                                  out.ctypes.data_as(C.POINTER(C.c_int32)))
    return out[:nb]


def nodal_mass(coords, conn, density, area):
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    m = np.zeros(coords.shape[0])
    lib().orc_nodal_mass(coords.shape[0], dptr(coords), conn.shape[0],
                         conn.ctypes.data_as(C.POINTER(C.c_int32)), density, area, dptr(m))
    return m


def scale_conversion(coords, conn, fiber_radius, volume_fraction):
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    return lib().orc_scale_conversion(coords.shape[0], dptr(coords), conn.shape[0],
                                      conn.ctypes.data_as(C.POINTER(C.c_int32)),
                                      float(fiber_radius), float(volume_fraction))
