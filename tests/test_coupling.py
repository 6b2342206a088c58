"""Host side of the macro/micro coupling front-end (no GPU): the scale
conversion against the oracle and a closed form, argument checks, and the
solver-record mapping."""
import numpy as np
import pytest

from conftest import network_2_7


@pytest.fixture(scope="module")
def CP(lib_path):
    from mumfim_gb300 import coupling
    return coupling


def test_scale_conversion_matches_oracle(CP, oracle, golden_2_7):
    from mumfim_gb300 import synthetic as S
    from mumfim_gb300.network_io import FiberNetwork
    nets = [network_2_7(golden_2_7)]
    for seed in (1, 2):
        coords, conn = S.knn_network(900, 4, S.geometry_seed(9, seed))
        nets.append(FiberNetwork(coords, conn))
    for net in nets:
        for r, vf in ((1e-3, 0.05), (3.5e-2, 0.4)):
            got = CP.scale_conversion(net, r, vf)
            want = oracle.scale_conversion(net.coords, net.connectivity, r, vf)
            assert got == want


def test_scale_conversion_closed_form(CP):
    from mumfim_gb300.network_io import FiberNetwork
    # one fiber of length 2: d^2 = L pi r^2 / vf, factor = vf / (2 pi r^2)
    net = FiberNetwork(np.array([[0.0, 0, 0], [2.0, 0, 0]]), np.array([[0, 1]], dtype=np.int32))
    r, vf = 0.01, 0.3
    assert CP.scale_conversion(net, r, vf) == pytest.approx(vf / (2 * np.pi * r * r), rel=1e-14)


def test_scale_conversion_rejects_bad_input(CP):
    from mumfim_gb300.batched import MumfimGpuError
    from mumfim_gb300.network_io import FiberNetwork
    net = FiberNetwork(np.array([[0.0, 0, 0], [1.0, 0, 0]]), np.array([[0, 1]], dtype=np.int32))
    for r, vf in ((0.0, 0.1), (1e-3, 0.0), (-1.0, 0.1), (np.nan, 0.1)):
        with pytest.raises(MumfimGpuError):
            CP.scale_conversion(net, r, vf)
    bad = FiberNetwork(net.coords, np.array([[0, 2]], dtype=np.int32))
    with pytest.raises(MumfimGpuError, match="out of range"):
        CP.scale_conversion(bad, 1e-3, 0.1)
    zero = FiberNetwork(np.zeros((2, 3)), np.array([[0, 1]], dtype=np.int32))
    with pytest.raises(MumfimGpuError):
        CP.scale_conversion(zero, 1e-3, 0.1)


def test_strategy_from_solver_fields(CP):
    rec = np.zeros(CP.NUM_MICRO_SOLVER_FIELDS)
    rec[CP.VISCOUS_DAMPING_FACTOR] = 0.7
    rec[CP.CRITICAL_TIME_SCALE_FACTOR] = 0.3  # ignored by the batched kernels
    s = CP.strategy_from_solver_fields(rec)
    assert s.visc_damp_coeff == 0.7
    assert s.crit_time_scale_factor == 0.8
    assert s.residual_tol == 1e-6 and s.max_steps == 0
