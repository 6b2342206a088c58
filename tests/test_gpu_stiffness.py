"""Material stiffness: the six perturbed solves run concurrently.

The reference runs the six perturbed, non-updating solves of the FD
stiffness one after the other over the whole batch
(BatchedFiberRVEAnalysisExplicit.h:321-405). The concurrent form keeps six
sets of per-solve scratch and runs all of them at once, each from the state
of the last updating run.
  - RAMP mode: the result is the sequential one bit for bit (stiffness,
    displacements and current coordinates), in both precisions.
  - RELAX mode: the reference's sequential runs chain through the current
    coordinates that each non-updating run leaves behind. The concurrent
    form equals, bit for bit, six runs that each restart from the exported
    state of the last updating run, and stays within the relaxation's
    tolerance of the chained order.
  - Mixed precision against FP64: the FD step h = 1e-5 divides the stress
    difference of each perturbed solve by h, but the mixed path's error is
    nearly the same in the base and the perturbed solves (same network, same
    state, nearly the same F), so it cancels: measured at most 3.8e-6 of the
    Frobenius norm per RVE on this batch; the bound here is 1e-4.
"""
import numpy as np
import pytest

from conftest import network_2_7

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(lib_path):
    import mumfim_gb300 as m
    return m


@pytest.fixture(scope="module")
def W(lib_path):
    from mumfim_gb300 import synthetic as S
    return S.config2(n_rve=10, steps=700, n_min=500, n_max=14_000)


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_concurrent_equals_sequential_in_ramp_mode(M, W, precision):
    out = {}
    for mode in ("sequential", "concurrent"):
        g = M.BatchedFiberRVEAnalysisExplicit(W.networks, W.strategies, precision=precision,
                                              stiffness=mode)
        s = np.zeros((W.n_rve, 6))
        g.run(W.F, s, update_coords=True)
        C = g.computeMaterialStiffness()
        out[mode] = (s, C, [g.displacements(r) for r in range(W.n_rve)],
                     [g.coordinates(r) for r in range(W.n_rve)], g.last_launches())
    (s0, C0, u0, x0, _), (s1, C1, u1, x1, launches) = out["sequential"], out["concurrent"]
    np.testing.assert_array_equal(s0, s1)
    np.testing.assert_array_equal(C0, C1)
    for r in range(W.n_rve):
        np.testing.assert_array_equal(u0[r], u1[r])
        np.testing.assert_array_equal(x0[r], x1[r])
    assert np.isfinite(C1).all() and np.abs(C1).max() > 0
    assert launches >= 6


def test_auto_is_concurrent_for_ramp_batches(M, W):
    g = M.BatchedFiberRVEAnalysisExplicit(W.networks, W.strategies)
    g.run(W.F, update_coords=True)
    g.computeMaterialStiffness()
    assert g.last_launches() == 6  # six concurrent FP64 launches, not one per sequential run


def test_relax_mode_concurrent_restarts_from_the_updated_state(M, golden_2_7):
    """RELAX mode on Network_2_7 (and a transposed-F copy): the concurrent
    stiffness equals six solves that each start from the exported state of
    the last updating run; the reference's chained order differs only at
    the level the relaxation tolerance allows."""
    g = golden_2_7
    nets = [network_2_7(g), network_2_7(g)]
    strat = [M.SolutionStrategy(visc_damp_coeff=g["visc_damp_coeff"], residual_tol=1e-6)] * 2
    F0 = np.array(g["F"]).reshape(3, 3)
    F = np.stack([F0, F0.T])
    conc = M.BatchedFiberRVEAnalysisExplicit(nets, strat, stiffness="concurrent")
    seq = M.BatchedFiberRVEAnalysisExplicit(nets, strat, stiffness="sequential")
    emu = M.BatchedFiberRVEAnalysisExplicit(nets, strat)
    for b in (conc, seq, emu):
        assert b.run(F, update_coords=True)
    C_conc = conc.computeMaterialStiffness()
    C_seq = seq.computeMaterialStiffness()
    # emulation: each perturbed solve from the exported updated state
    state = [emu.export_state(r) for r in range(2)]
    cur = emu.current_stress()
    h = 1e-5
    C_emu = np.zeros((2, 6, 6))
    from mumfim_gb300 import _abi  # noqa: F401
    Fa = _perturbations()
    for i in range(6):
        for r in range(2):
            emu.import_state(r, state[r])
        s = np.zeros((2, 6))
        emu.run(Fa[i][None], s, update_coords=False)
        C_emu[:, :, i] = (s - cur) / h
    np.testing.assert_array_equal(C_conc, C_emu)
    rel = np.linalg.norm(C_conc - C_seq) / np.linalg.norm(C_seq)
    assert rel <= 1e-2, rel


def _perturbations():
    """The six perturbation gradients, h = 1e-5, in the library's (and the
    reference's) arithmetic order."""
    import math
    h = 1e-5
    D1 = math.sqrt(1.0 / (1 - 2 * h))
    l1 = 1.0
    l2 = (1 + h) / (1 - h * h)
    l3 = (1 - h) / (1 - h * h)
    p = 0.5 * (math.sqrt(l2) + math.sqrt(l3))
    q = 0.5 * (math.sqrt(l2) - math.sqrt(l3))
    out = []
    for i in range(6):
        F = np.zeros((3, 3))
        if i < 3:
            F[0, 0] = F[1, 1] = F[2, 2] = 1.0
            F[i, i] = D1
        elif i == 3:
            F[0, 0], F[1, 1], F[2, 2], F[1, 2], F[2, 1] = l1, p, p, q, q
        elif i == 4:
            F[0, 0], F[1, 1], F[2, 2], F[0, 2], F[2, 0] = p, l1, p, q, q
        else:
            F[0, 0], F[1, 1], F[2, 2], F[0, 1], F[1, 0] = p, p, l1, q, q
        out.append(F)
    return out


def test_mixed_stiffness_against_fp64(M, W):
    """States the mixed path's stiffness error against FP64 (RAMP mode, the
    concurrent form in both): within 1e-4 of the Frobenius norm per RVE."""
    C = {}
    for prec in ("f64", "mixed"):
        g = M.BatchedFiberRVEAnalysisExplicit(W.networks, W.strategies, precision=prec)
        g.run(W.F, update_coords=True)
        C[prec] = g.computeMaterialStiffness()
    err = (np.linalg.norm((C["mixed"] - C["f64"]).reshape(W.n_rve, -1), axis=1)
           / np.linalg.norm(C["f64"].reshape(W.n_rve, -1), axis=1))
    print("mixed vs FP64 stiffness, relative Frobenius error per RVE:", err.tolist())
    assert err.max() <= 1e-4, err
