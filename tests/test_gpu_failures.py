"""Failure detection on the GPU, with failures made on the host.

No test here faults, traps or hangs the GPU. A bad input is planted in the
deformation gradients the host passes in (NaN, Inf, or finite values so
large that the solve overflows); the kernels must report MFG_E_NONFINITE for
that RVE and leave every other RVE's result bit-identical to a clean run.
The reference's loop has no such check: it leaves its relaxation loop
silently on a NaN residual
(BatchedFiberRVEAnalysisExplicitTeamOuterLoop.h:340-371). The server's waits
are made to run out on purpose: a host-side poll limit, and the persistent
kernel's bound on one device-side wait.
"""
import ctypes as C
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MFG_E_NONFINITE = 4
MFG_E_TIMEOUT = 5


@pytest.fixture(scope="module")
def W(lib_path):
    from mumfim_gb300 import synthetic as S
    return S.config2(n_rve=6, steps=600, n_min=500, n_max=9_000)


@pytest.mark.parametrize("precision", ["f64", "mixed"])
@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_nonfinite_F_flags_only_its_rve(W, precision, bad):
    import mumfim_gb300 as m
    clean = m.BatchedFiberRVEAnalysisExplicit(W.networks, W.strategies, precision=precision)
    s_clean = np.zeros((W.n_rve, 6))
    assert clean.run(W.F, s_clean, update_coords=False)
    F = W.F.copy()
    F[2, 1, 0] = bad
    g = m.BatchedFiberRVEAnalysisExplicit(W.networks, W.strategies, precision=precision)
    s = np.zeros((W.n_rve, 6))
    ok = g.run(F, s, update_coords=False)
    assert not ok
    st = g.last_status["status"]
    assert st[2] == MFG_E_NONFINITE
    others = [r for r in range(W.n_rve) if r != 2]
    assert (st[others] == 0).all()
    np.testing.assert_array_equal(s[others], s_clean[others])


def test_relax_mode_nonfinite_F(lib_path):
    """RELAX mode (affine predictor, residual loop): a NaN increment ends that
    RVE's loop at its first residual check with MFG_E_NONFINITE."""
    import mumfim_gb300 as m
    from mumfim_gb300 import synthetic as S
    w = S.config1(n_rve=3, n_nodes=600)
    strat = [m.SolutionStrategy(visc_damp_coeff=2.0, residual_tol=1e-9, max_steps=3000)] * 3
    F = w.F.copy()
    F[0, 0, 0] = np.nan
    for prec in ("f64", "mixed"):
        g = m.BatchedFiberRVEAnalysisExplicit(w.networks, strat, precision=prec)
        ref = m.BatchedFiberRVEAnalysisExplicit(w.networks, strat, precision=prec)
        s, s_ref = np.zeros((3, 6)), np.zeros((3, 6))
        g.run(F, s, update_coords=True)
        ref.run(w.F, s_ref, update_coords=True)
        assert g.last_status["status"][0] == MFG_E_NONFINITE
        assert g.last_status["steps"][0] <= 101
        np.testing.assert_array_equal(s[1:], s_ref[1:])
        np.testing.assert_array_equal(g.last_status[1:], ref.last_status[1:])


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_server_overflowing_request_flags_only_itself(W, precision):
    """A finite F far too large to solve overflows inside the kernel: that
    request comes back MFG_E_NONFINITE while the requests in flight with it
    give the clean results. A non-finite F is refused at submission."""
    import mumfim_gb300 as m
    from mumfim_gb300.serving import RVEServer
    ref = m.BatchedFiberRVEAnalysisExplicit(W.networks, W.strategies, precision=precision)
    s_ref = np.zeros((W.n_rve, 6))
    ref.run(W.F, s_ref, update_coords=False)
    with RVEServer(W.networks, W.strategies, precision=precision) as sv:
        with pytest.raises(m.MumfimGpuError) as ei:
            sv.submit(1, np.full((3, 3), np.nan), update_coords=False)
        assert ei.value.status == 1
        for r in range(W.n_rve):
            F = np.full((3, 3), 1e300) if r == 4 else W.F[r]
            sv.submit(r, F, update_coords=False)
        res = sv.drain()
    assert len(res) == W.n_rve
    for rec in res:
        if rec["rve"] == 4:
            assert rec["status"] == MFG_E_NONFINITE
        else:
            assert rec["status"] == 0
            np.testing.assert_array_equal(rec["sigma"], s_ref[rec["rve"]])


def test_server_poll_times_out(lib_path):
    """mfg_server_poll returns MFG_E_TIMEOUT when work is outstanding and
    nothing completes within its limit; the result arrives later."""
    import mumfim_gb300 as m
    from mumfim_gb300 import synthetic as S
    from mumfim_gb300.serving import RVEServer
    coords, conn = S.knn_network(6_000, 4, S.geometry_seed(21, 0))
    net = m.FiberNetwork(coords, conn, [S._linear_params(21, 0)])
    strat = m.SolutionStrategy.ramp(5_000, 0.5)  # about 0.1 s on one CTA
    with RVEServer([net], [strat], precision="mixed") as sv:
        sv.submit(0, np.eye(3) + 0.01 * np.eye(3), update_coords=False)
        res, rc = sv.poll_status(timeout_ms=1)
        assert rc == MFG_E_TIMEOUT and len(res) == 0
        L = m.load_library()
        assert "no request completed" in L.mfg_last_error().decode()
        res = sv.drain()
        assert len(res) == 1 and res["status"][0] == 0


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_server_kernel_leaves_after_its_wait_bound(W, precision):
    """With the collective idle shutdown pushed out to 30 s, the persistent
    kernel still frees the SMs once each CTA has waited max_wait_ms without
    work: a later request needs a fresh launch. (The mixed-precision server
    of this batch runs the 4-CTA cluster kernel, the FP64 one the per-CTA
    loop.)"""
    from mumfim_gb300.serving import RVEServer
    with RVEServer(W.networks, W.strategies, precision=precision, idle_timeout_us=30_000_000,
                   max_wait_ms=100) as sv:
        sv.submit(0, W.F[0], update_coords=False)
        assert len(sv.drain()) == 1
        assert sv.launches() == 1
        time.sleep(1.0)
        sv.submit(1, W.F[1], update_coords=False)
        assert len(sv.drain()) == 1
        assert sv.launches() == 2
