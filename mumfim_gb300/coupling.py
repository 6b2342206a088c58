"""Macro/micro coupling front-end of the batched solve.

Mirrors what the multiscale service does around the batched analysis
(src/mumfim/microscale/MultiscaleRVEAnalysis.cc:137-305):

* at set-up, every fiber network gets the scale conversion of
  ``calcScaleConversion`` (MultiscaleCoupling.cc:7-23) from its
  ``micro_fo_params`` record (fiber radius, volume fraction), and every RVE a
  solution strategy from its solver records (``serializeSolutionStrategy``,
  MultiscaleRVEAnalysis.cc:306-334);
* each macro iteration takes ``micro_fo_data`` records (F, row-major) and
  returns ``micro_fo_result`` records: stress (6), averaged volume stress (3,
  zero as in the reference) and the 6 x 6 stiffness (36);
* each load step returns ``micro_fo_step_result`` records: the 3-D
  orientation tensor (9) and the 2-D one about the record's orientation axis
  (9), as ``recoverMultiscaleStepResults`` (MultiscaleCoupling.h:46-66).

Record layouts are those of MultiscaleMicroFOParams.h:33-104.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from ._abi import MFG_E_NOT_CONVERGED, MFG_OK, RVE_STATUS_DTYPE, dptr
from .batched import BatchedFiberRVEAnalysisExplicit, _check, load_library
from .network_io import FiberNetwork
from .strategy import SolutionStrategy

# fiber_param_fields (MultiscaleMicroFOParams.h:33-44)
FIBER_RADIUS, VOLUME_FRACTION, YOUNGS_MODULUS, NONLINEAR_PARAM, LINEAR_TRANSITION = range(5)
ORIENTATION_AXIS_X, ORIENTATION_AXIS_Y, ORIENTATION_AXIS_Z = 5, 6, 7
NUM_PARAM_FIELDS = 8
# micro_solver_fields (MultiscaleMicroFOParams.h:45-56)
(MICRO_SOLVER_TOL, MICRO_CONVERGENCE_TOL, PREV_ITER_FACTOR, LOAD_TIME, HOLD_TIME,
 VISCOUS_DAMPING_FACTOR, CRITICAL_TIME_SCALE_FACTOR, ENERGY_CHECK_EPSILON) = range(8)
NUM_MICRO_SOLVER_FIELDS = 8

MICRO_FO_DATA = 9
MICRO_FO_RESULT = 45
MICRO_FO_STEP_RESULT = 18


def _lib():
    L = load_library()
    if not getattr(L, "_coupling_ready", False):
        vp, i32, dp = C.c_void_p, C.c_int32, C.POINTER(C.c_double)
        L.mfg_scale_conversion.restype = i32
        L.mfg_scale_conversion.argtypes = [i32, dp, i32, C.POINTER(i32), C.c_double, C.c_double,
                                           dp]
        L.mfg_batch_micro_fo_iterate.restype = i32
        L.mfg_batch_micro_fo_iterate.argtypes = [vp, dp, dp, vp]
        L.mfg_batch_micro_fo_step.restype = i32
        L.mfg_batch_micro_fo_step.argtypes = [vp, dp, dp]
        L._coupling_ready = True
    return L


def scale_conversion(network: FiberNetwork, fiber_radius: float, volume_fraction: float) -> float:
    """1 / d^2 with d = sqrt(L pi r^2 / volume_fraction), L the summed fiber
    length of the network (MultiscaleCoupling.cc:7-23)."""
    coords = np.ascontiguousarray(network.coords, dtype=np.float64)
    conn = np.ascontiguousarray(network.connectivity, dtype=np.int32)
    out = C.c_double()
    _check(_lib().mfg_scale_conversion(coords.shape[0], dptr(coords), conn.shape[0],
                                       conn.ctypes.data_as(C.POINTER(C.c_int32)),
                                       float(fiber_radius), float(volume_fraction),
                                       C.byref(out)))
    return out.value


def strategy_from_solver_fields(solver: Sequence[float]) -> SolutionStrategy:
    """Explicit strategy of one RVE from its micro_fo_solver record
    (serializeSolutionStrategy, MultiscaleRVEAnalysis.cc:306-334). The batched
    reference kernels read only the damping; they fix the critical-step
    factor at 0.8 (BatchedFiberRVEAnalysisExplicitTeamOuterLoop.h:312) and
    relax to a residual of 1e-6, whatever the record says, and so does this."""
    return SolutionStrategy(visc_damp_coeff=float(solver[VISCOUS_DAMPING_FACTOR]),
                            crit_time_scale_factor=0.8, residual_tol=1e-6)


class MicroFOBatch:
    """The batched microscale side of the multiscale exchange.

    networks  sequence of FiberNetwork; their scale_factor is set from params
    params    (n_rve, 8) micro_fo_params records
    strategies  one SolutionStrategy per RVE (strategy_from_solver_fields
                builds them from micro_fo_solver records)
    """

    def __init__(self, networks: Sequence[FiberNetwork], params, strategies: Sequence,
                 precision: str = "f64", device: int = 0):
        self.params = np.ascontiguousarray(params, dtype=np.float64).reshape(-1, NUM_PARAM_FIELDS)
        if self.params.shape[0] != len(networks):
            raise ValueError("one micro_fo_params record per network")
        for net, prm in zip(networks, self.params):
            net.scale_factor = scale_conversion(net, prm[FIBER_RADIUS], prm[VOLUME_FRACTION])
        self.analysis = BatchedFiberRVEAnalysisExplicit(networks, strategies, precision=precision,
                                                        device=device)
        self.n_rve = len(networks)
        self.last_status = np.zeros(self.n_rve, dtype=RVE_STATUS_DTYPE)

    def close(self):
        self.analysis.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def iterate(self, data) -> np.ndarray:
        """One macro iteration: (n_rve, 9) micro_fo_data in, (n_rve, 45)
        micro_fo_result out. RVEs that did not converge are reported in
        last_status, as the reference's run() reports them by its return."""
        data = np.ascontiguousarray(data, dtype=np.float64).reshape(self.n_rve, MICRO_FO_DATA)
        out = np.zeros((self.n_rve, MICRO_FO_RESULT))
        st = np.zeros(self.n_rve, dtype=RVE_STATUS_DTYPE)
        _check(_lib().mfg_batch_micro_fo_iterate(self.analysis.handle, dptr(data), dptr(out),
                                                  st.ctypes.data_as(C.c_void_p)),
               allow=(MFG_OK, MFG_E_NOT_CONVERGED))
        self.last_status = st
        return out

    def step_results(self) -> np.ndarray:
        """(n_rve, 18) micro_fo_step_result records of the current state."""
        out = np.zeros((self.n_rve, MICRO_FO_STEP_RESULT))
        _check(_lib().mfg_batch_micro_fo_step(self.analysis.handle, dptr(self.params), dptr(out)))
        return out
