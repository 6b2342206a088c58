"""FP64 GPU kernel vs the CPU oracle, through the C ABI.

The plain FP64 kernel restates the reference's operation order without
contraction and gathers nodal forces in the serial scatter order, so for the
linear law its displacements, stresses and step counts must be
bit-identical to the oracle's. The nonlinear law calls exp(), whose device
and host implementations may differ in the last bit: tolerance 1e-10
relative there, as for any FP64 result.
"""
import numpy as np
import pytest

from conftest import network_2_7, voigt_to_mat

pytestmark = pytest.mark.gpu

REL_F64 = 1e-10


def _rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def M(lib_path):
    import mumfim_gb300 as m
    return m


def _pair(M, oracle, nets, strats, precision="f64"):
    return (M.BatchedFiberRVEAnalysisExplicit(nets, strats, precision=precision),
            oracle.OracleBatch(nets, strats))


def test_network_2_7_relax_bitwise_and_golden(M, oracle, golden_2_7):
    g = golden_2_7
    net = network_2_7(g)
    s = M.SolutionStrategy(visc_damp_coeff=g["visc_damp_coeff"], crit_time_scale_factor=0.8,
                           residual_tol=1e-6)
    gpu, orc = _pair(M, oracle, [net], [s])
    F = np.array(g["F"]).reshape(1, 3, 3)
    sig = np.zeros((1, 6))
    assert gpu.run(F, sig)
    rc, sig_o, st_o = orc.run(F)
    assert rc == 0
    assert gpu.last_status["steps"][0] == st_o["steps"][0]
    assert gpu.last_status["status"][0] == 0
    np.testing.assert_array_equal(sig, sig_o)
    np.testing.assert_array_equal(gpu.displacements(0), orc.displacements(0))
    np.testing.assert_array_equal(gpu.coordinates(0), orc.coordinates(0))
    assert abs(gpu.last_status["residual"][0] - st_o["residual"][0]) <= 1e-12 * st_o["residual"][0]
    # the reference's own printed stress (legacy explicit solver, no 1/V)
    J = np.linalg.det(F[0])
    gold = np.array(g["outputs"]["explicit_cpu_out"]["stress"][0])
    assert np.abs(voigt_to_mat(sig[0] * J) - gold).max() <= 1e-5 * np.abs(gold).max()


def test_material_stiffness_bitwise(M, oracle, golden_2_7):
    g = golden_2_7
    net = network_2_7(g)
    s = M.SolutionStrategy(visc_damp_coeff=g["visc_damp_coeff"], residual_tol=1e-6)
    gpu, orc = _pair(M, oracle, [net], [s])
    F = np.array(g["F"]).reshape(1, 3, 3)
    gpu.run(F)
    orc.run(F)
    Cg = gpu.computeMaterialStiffness()
    rc, Co = orc.material_stiffness()
    np.testing.assert_array_equal(Cg, Co)
    np.testing.assert_array_equal(gpu.displacements(0), orc.displacements(0))
    np.testing.assert_array_equal(gpu.coordinates(0), orc.coordinates(0))
    gold = np.array(g["outputs"]["explicit_cpu_out"]["stiffness"][0])
    assert np.linalg.norm(Cg[0] - gold) <= 0.05 * np.linalg.norm(gold)


def test_config0_ramp_bitwise(M, oracle):
    from mumfim_gb300 import synthetic as S
    w = S.config0(steps=10_000)
    gpu, orc = _pair(M, oracle, w.networks, w.strategies)
    sig = np.zeros((1, 6))
    gpu.run(w.F, sig)
    rc, sig_o, st_o = orc.run(w.F)
    assert gpu.last_status["steps"][0] == 10_000 == st_o["steps"][0]
    np.testing.assert_array_equal(sig, sig_o)
    np.testing.assert_array_equal(gpu.displacements(0), orc.displacements(0))


def test_config1_subset_bitwise(M, oracle):
    from mumfim_gb300 import synthetic as S
    w = S.config1(n_rve=16, steps=5_000)
    gpu, orc = _pair(M, oracle, w.networks, w.strategies)
    sig = np.zeros((16, 6))
    gpu.run(w.F, sig)
    rc, sig_o, st_o = orc.run(w.F, n_threads=16)
    np.testing.assert_array_equal(gpu.last_status["steps"], st_o["steps"])
    np.testing.assert_array_equal(sig, sig_o)
    for r in (0, 7, 15):
        np.testing.assert_array_equal(gpu.displacements(r), orc.displacements(r))


def test_incremental_runs_and_transactional_run(M, oracle):
    """Two updating runs (incremental F on the current configuration), then a
    non-updating run: u is restored, x keeps the perturbed solve (the
    reference's quirk), and the next updating run starts from there."""
    from mumfim_gb300 import synthetic as S
    w = S.config1(n_rve=3, n_nodes=600)
    strat = [M.SolutionStrategy(visc_damp_coeff=2.0, residual_tol=1e-9, max_steps=3000)
             for _ in range(3)]
    gpu, orc = _pair(M, oracle, w.networks, strat)
    F1 = w.F
    F2 = np.repeat(np.eye(3)[None] + 0.01 * np.array([[0, 1, 0], [0, 0, 0], [0, 0, -1.0]]), 3, 0)
    for F, upd in ((F1, True), (F2, True), (F2[:1], False), (F1, True)):
        sig = np.zeros((3, 6))
        gpu.run(F, sig, update_coords=upd)
        rc, sig_o, st_o = orc.run(F, update_coords=upd)
        np.testing.assert_array_equal(sig, sig_o)
        np.testing.assert_array_equal(gpu.last_status["steps"], st_o["steps"])
        np.testing.assert_array_equal(gpu.last_status["status"], st_o["status"])
        for r in range(3):
            np.testing.assert_array_equal(gpu.displacements(r), orc.displacements(r))
            np.testing.assert_array_equal(gpu.coordinates(r), orc.coordinates(r))
    np.testing.assert_array_equal(gpu.current_stress(), orc.current_stress())


def test_step_cap_reports_not_converged(M, oracle):
    from mumfim_gb300 import synthetic as S
    w = S.config1(n_rve=2, n_nodes=500)
    strat = [M.SolutionStrategy(visc_damp_coeff=0.5, residual_tol=1e-30, max_steps=250)] * 2
    gpu, orc = _pair(M, oracle, w.networks, strat)
    ok = gpu.run(w.F)
    assert not ok
    assert list(gpu.last_status["status"]) == [3, 3]
    assert list(gpu.last_status["steps"]) == [250, 250]
    rc, sig_o, st_o = orc.run(w.F)
    np.testing.assert_array_equal(gpu.last_sigma, sig_o)


def test_nonlinear_law(M, oracle):
    from mumfim_gb300 import synthetic as S
    w = S.config3(n_rve=4, steps=2_000, n_min=400, n_max=900)
    gpu, orc = _pair(M, oracle, w.networks, w.strategies)
    sig = np.zeros((4, 6))
    gpu.run(w.F, sig)
    rc, sig_o, st_o = orc.run(w.F, n_threads=4)
    assert _rel(sig, sig_o) <= REL_F64
    for r in range(4):
        assert _rel(gpu.displacements(r), orc.displacements(r)) <= REL_F64


def test_orientation_tensors(M, oracle):
    from mumfim_gb300 import synthetic as S
    w = S.config1(n_rve=3, n_nodes=700, steps=300)
    gpu, orc = _pair(M, oracle, w.networks, w.strategies)
    np.testing.assert_allclose(gpu.compute3DOrientationTensor(), orc.orientation_3d(),
                               rtol=0, atol=1e-14)
    gpu.run(w.F)
    orc.run(w.F)
    normal = np.array([[1.0, 0, 0], [0, 2.0, 0], [0.3, 0.4, 0.5]])
    np.testing.assert_allclose(gpu.compute3DOrientationTensor(), orc.orientation_3d(),
                               rtol=0, atol=1e-14)
    np.testing.assert_allclose(gpu.compute2DOrientationTensor(normal), orc.orientation_2d(normal),
                               rtol=0, atol=1e-14)


def test_export_import_state_round_trip(M, oracle):
    from mumfim_gb300 import synthetic as S
    w = S.config1(n_rve=2, n_nodes=500, steps=400)
    a = M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies)
    b = M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies)
    a.run(w.F)
    for r in range(2):
        b.import_state(r, a.export_state(r))
    sa, sb = np.zeros((2, 6)), np.zeros((2, 6))
    a.run(w.F, sa)
    b.run(w.F, sb)
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(a.displacements(1), b.displacements(1))


def test_invalid_arguments_raise(M):
    from mumfim_gb300 import synthetic as S
    w = S.config1(n_rve=2, n_nodes=300, steps=100)
    gpu = M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies)
    with pytest.raises(M.MumfimGpuError) as ei:
        gpu.run(w.F[:1], update_coords=True)  # broadcast F only without update
    assert ei.value.status == 1
    with pytest.raises(M.MumfimGpuError):
        gpu.run(np.zeros((3, 3, 3)))
