"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the mumfim_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from mumfim_gb300._abi import (NetworkArray, RVE_STATUS_DTYPE, dptr, mfg_network,
                               mfg_rve_status, mfg_strategy)

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    """Compiles the oracle (-O2 -ffp-contract=off, no -march so x86-64 and
    aarch64 give the same bits)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "mumfim_oracle.cpp")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "mumfim_oracle.h"))):
        return LIB_PATH
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
           "-I" + os.path.join(REPO, "include"), "-I" + HERE, src, "-o", LIB_PATH + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
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
        _lib = L
    return _lib


class OracleBatch:
    """CPU restatement of BatchedFiberRVEAnalysisExplicit with the same
    arguments as mumfim_gb300.BatchedFiberRVEAnalysisExplicit."""

    def __init__(self, networks, strategies):
        self._arr = NetworkArray(networks, strategies)
        self.n_rve = len(networks)
        self.n_nodes = [n.n_nodes for n in networks]
        self._h = lib().orc_batch_create(self._arr.nets, self._arr.strats, self.n_rve)
        if not self._h:
            raise ValueError("oracle rejected the networks")

    def close(self):
        if self._h:
            lib().orc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def run(self, F, update_coords=True, n_threads=1):
        F = np.ascontiguousarray(F, dtype=np.float64).reshape(-1, 9)
        sigma = np.zeros((self.n_rve, 6))
        st = np.zeros(self.n_rve, dtype=RVE_STATUS_DTYPE)
        rc = lib().orc_batch_run(self._h, dptr(F), F.shape[0], dptr(sigma), int(update_coords),
                                 st.ctypes.data_as(C.c_void_p), n_threads)
        return rc, sigma, st

    def material_stiffness(self, n_threads=1):
        Cm = np.zeros((self.n_rve, 6, 6))
        rc = lib().orc_batch_material_stiffness(self._h, dptr(Cm), n_threads)
        return rc, Cm

    def orientation_3d(self):
        om = np.zeros((self.n_rve, 3, 3))
        lib().orc_batch_orientation_3d(self._h, dptr(om))
        return om

    def orientation_2d(self, normal):
        normal = np.ascontiguousarray(normal, dtype=np.float64).reshape(self.n_rve, 3)
        om = np.zeros((self.n_rve, 3, 3))
        lib().orc_batch_orientation_2d(self._h, dptr(normal), dptr(om))
        return om

    def displacements(self, rve):
        u = np.zeros((self.n_nodes[rve], 3))
        lib().orc_batch_get_displacements(self._h, rve, dptr(u))
        return u

    def coordinates(self, rve):
        x = np.zeros((self.n_nodes[rve], 3))
        lib().orc_batch_get_coordinates(self._h, rve, dptr(x))
        return x

    def current_stress(self):
        s = np.zeros((self.n_rve, 6))
        lib().orc_batch_get_current_stress(self._h, dptr(s))
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
