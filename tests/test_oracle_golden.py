"""The CPU oracle against the reference's own known answers (no GPU)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, network_2_7, voigt_to_mat


def _strategy(g, **kw):
    from mumfim_gb300 import SolutionStrategy
    return SolutionStrategy(visc_damp_coeff=g["visc_damp_coeff"], crit_time_scale_factor=0.8,
                            residual_tol=1e-6, **kw)


@pytest.fixture(scope="module")
def solved_2_7(oracle, golden_2_7):
    g = golden_2_7
    b = oracle.OracleBatch([network_2_7(g)], [_strategy(g)])
    F = np.array(g["F"]).reshape(1, 3, 3)
    rc, sig, st = b.run(F)
    return g, b, F, rc, sig, st


def test_network_2_7_stress_matches_reference_outputs(solved_2_7):
    g, b, F, rc, sig, st = solved_2_7
    assert rc == 0 and st["status"][0] == 0
    assert st["steps"][0] % 100 == 1  # the loop only stops right after a residual refresh
    assert st["residual"][0] <= 1e-6
    J = np.linalg.det(F[0])
    # The legacy solvers print stress without the batched path's 1/V factor.
    for name in ("explicit_cpu_out", "explicit_gpu_out", "implicit_out"):
        gold = np.array(g["outputs"][name]["stress"][0])
        err = np.abs(voigt_to_mat(sig[0] * J) - gold).max() / np.abs(gold).max()
        assert err <= 1e-5, (name, err)


def test_network_2_7_stiffness_matches_reference_outputs(solved_2_7):
    g, b, F, rc, sig, st = solved_2_7
    rc, C = b.material_stiffness()
    for name in ("explicit_cpu_out", "explicit_gpu_out"):
        for gold in g["outputs"][name]["stiffness"]:
            gold = np.array(gold)
            assert np.linalg.norm(C[0] - gold) <= 0.05 * np.linalg.norm(gold)
    # the non-updating runs leave u and the stress of the last updating run alone
    np.testing.assert_array_equal(b.current_stress(), sig)


def test_reorder_known_answer(oracle):
    with open(os.path.join(GOLDEN, "reorder_kat.json")) as fh:
        kat = json.load(fh)
    perm = oracle.reorder_permutation(kat["n_verts"], kat["fixed_verts"])
    conn = np.array(kat["initial_connectivity"])
    assert perm[conn].tolist() == kat["final_connectivity"]
    coords = np.arange(3 * kat["n_verts"], dtype=float).reshape(-1, 3)
    out = np.zeros_like(coords)
    out[perm] = coords
    assert out.reshape(-1).tolist() == kat["final_coordinates"]


def test_boundary_nodes_follow_rve_cube_faces(oracle):
    c = np.array([[0.0, 0.0, 0.0], [0.5, 0.1, 0.1], [-0.5, 0, 0], [0.1, 0.5 - 5e-9, 0.2],
                  [0.1, 0.5 - 2e-8, 0.2], [0.2, 0.3, -0.5], [0.49999, 0.49999, 0.49999]])
    assert oracle.boundary_nodes(c).tolist() == [1, 2, 3, 5]


def test_lumped_mass_of_a_chain(oracle):
    c = np.array([[0.0, 0, 0], [0.3, 0, 0], [0.3, 0.4, 0]])
    conn = np.array([[0, 1], [1, 2]], dtype=np.int32)
    rho, A = 7.0, 0.25
    m = oracle.nodal_mass(c, conn, rho, A)
    np.testing.assert_allclose(m, [rho * A * 0.3 / 2, rho * A * (0.3 + 0.4) / 2, rho * A * 0.4 / 2],
                               rtol=1e-15)


def test_affine_network_is_stress_free_and_exactly_mapped(oracle):
    """Size-independent property: if every node is on the boundary the RAMP
    solve is the affine map x = F x0 and, with a linear law, the stress is
    the fibers' sum of x (x) f."""
    from mumfim_gb300 import FiberNetwork, Reaction, SolutionStrategy
    c = np.array([[-0.5, -0.5, -0.5], [0.5, -0.5, -0.5], [0.5, 0.5, -0.5], [-0.5, 0.5, 0.5]])
    conn = np.array([[0, 1], [1, 2], [2, 3], [3, 0]], dtype=np.int32)
    net = FiberNetwork(c, conn, [Reaction(0, 0.1, 2.0, 1.0)])
    b = oracle.OracleBatch([net], [SolutionStrategy.ramp(7)])
    F = np.array([[1.1, 0.05, 0.0], [0.0, 0.95, 0.0], [0.0, 0.0, 1.0]])
    rc, sig, st = b.run(F.reshape(1, 9))
    x = b.coordinates(0)
    np.testing.assert_allclose(x, c @ F.T, rtol=0, atol=1e-15)
    # independent evaluation of sigma = (1/V) sum_b sym(x (x) f)
    A = 0.1 * 0.1 * np.pi
    f = np.zeros_like(c)
    for a_, b_ in conn:
        d = x[b_] - x[a_]
        l = np.linalg.norm(d)
        l0 = np.linalg.norm(c[b_] - c[a_])
        lam = l / l0
        T = lam * 2.0 * A * 0.5 * (lam * lam - 1)
        f[a_] -= d * T / l
        f[b_] += d * T / l
    S = sum(np.outer(x[i], f[i]) for i in range(4))
    S = 0.5 * (S + S.T) / np.linalg.det(F)
    np.testing.assert_allclose(voigt_to_mat(sig[0]), S, rtol=1e-12, atol=1e-15)


def test_transactional_run_restores_displacement(oracle, golden_2_7):
    g = golden_2_7
    b = oracle.OracleBatch([network_2_7(g)], [_strategy(g, max_steps=500)])
    F = np.array(g["F"]).reshape(1, 3, 3)
    b.run(F)
    u0 = b.displacements(0).copy()
    b.run(np.diag([1.01, 1, 1]).reshape(1, 3, 3), update_coords=False)
    np.testing.assert_array_equal(b.displacements(0), u0)


def test_timing_build_agrees_with_the_parity_build(oracle):
    """The CPU baseline times the oracle's optimised build (-O3, FMA
    contraction allowed); it must solve the same problem: stresses within
    1e-9 of the bit-stable parity build on a fixed-step case."""
    from mumfim_gb300 import synthetic as S
    w = S.config1(n_rve=3, n_nodes=500, steps=500)
    rc, sig, st = oracle.OracleBatch(w.networks, w.strategies).run(w.F, n_threads=3)
    rc_t, sig_t, st_t = oracle.OracleBatch(w.networks, w.strategies, timing=True).run(
        w.F, n_threads=3)
    assert rc == rc_t == 0
    np.testing.assert_array_equal(st["steps"], st_t["steps"])
    assert np.abs(sig_t - sig).max() <= 1e-9 * np.abs(sig).max()
