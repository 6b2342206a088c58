"""Parity at the benchmark configurations' full RVE sizes and step counts.

FP64 GPU kernel against the CPU oracle:
  - config 2's largest RVEs (12,000 - 20,000 nodes, k in {3, 4, 5}):
    bit-identical stresses, displacements and step counts (linear law);
  - config 3 (exponential-toe law, 2,000 - 8,000 nodes, stretch up to 1.25
    and shear up to 0.15, so most fibers cross the toe transition): within
    1e-10, the tolerance of every FP64 result that goes through exp();
    including one RVE at config 3's full 20,000 steps.
Mixed precision against the FP64 kernel (GPU only), within 1e-5 relative
stress error: config 3 at full size and 20,000 steps, and config 2's largest
RVEs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_F64 = 1e-10
REL_MIXED = 1e-5


def _rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def M(lib_path):
    import mumfim_gb300 as m
    return m


def _largest(w, count, lo):
    """Ids of the `count` largest RVEs with at least `lo` nodes."""
    ids = [r for r in np.argsort([-n.n_nodes for n in w.networks]) if w.networks[r].n_nodes >= lo]
    return sorted(int(r) for r in ids[:count])


@pytest.fixture(scope="module")
def config2_large(lib_path):
    from mumfim_gb300 import synthetic as S
    w = S.config2(n_rve=96, steps=1_000)  # the first 96 RVEs of config 2
    ids = _largest(w, 4, 12_000)
    assert len(ids) == 4
    return w.subset(ids)


def test_config2_largest_rves_fp64_bitwise(M, oracle, config2_large):
    w = config2_large
    assert min(n.n_nodes for n in w.networks) >= 12_000
    gpu = M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies)
    sig = np.zeros((w.n_rve, 6))
    gpu.run(w.F, sig, update_coords=True)
    orc = oracle.OracleBatch(w.networks, w.strategies)
    rc, sig_o, st_o = orc.run(w.F, n_threads=w.n_rve)
    np.testing.assert_array_equal(gpu.last_status["steps"], st_o["steps"])
    np.testing.assert_array_equal(sig, sig_o)
    for r in range(w.n_rve):
        np.testing.assert_array_equal(gpu.displacements(r), orc.displacements(r))


def test_config3_full_size_fp64_vs_oracle(M, oracle):
    from mumfim_gb300 import synthetic as S
    w = S.config3(n_rve=4, steps=4_000)
    assert max(n.n_nodes for n in w.networks) > 4_000
    gpu = M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies)
    sig = np.zeros((w.n_rve, 6))
    gpu.run(w.F, sig, update_coords=True)
    orc = oracle.OracleBatch(w.networks, w.strategies)
    rc, sig_o, st_o = orc.run(w.F, n_threads=w.n_rve)
    np.testing.assert_array_equal(gpu.last_status["steps"], st_o["steps"])
    assert _rel(sig, sig_o) <= REL_F64
    for r in range(w.n_rve):
        assert _rel(gpu.displacements(r), orc.displacements(r)) <= REL_F64


def test_config3_full_step_count_fp64_vs_oracle(M, oracle):
    """One config-3 RVE over the configuration's own 20,000 steps."""
    from mumfim_gb300 import synthetic as S
    w = S.config3(n_rve=8, steps=20_000)
    r = int(np.argmin([n.n_nodes for n in w.networks]))
    w = w.subset([r])
    gpu = M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies)
    sig = np.zeros((1, 6))
    gpu.run(w.F, sig)
    orc = oracle.OracleBatch(w.networks, w.strategies)
    rc, sig_o, st_o = orc.run(w.F)
    assert gpu.last_status["steps"][0] == st_o["steps"][0] == 20_000
    assert _rel(sig, sig_o) <= REL_F64
    assert _rel(gpu.displacements(0), orc.displacements(0)) <= REL_F64


def test_config3_full_size_mixed_vs_fp64(M):
    """Config 3 as specified (2,000 - 8,000 nodes, 20,000 steps) on 8 RVEs:
    the mixed-precision stress within 1e-5 of the FP64 kernel's."""
    from mumfim_gb300 import synthetic as S
    w = S.config3(n_rve=8)
    assert w.steps == 20_000
    out = {}
    for prec in ("f64", "mixed"):
        g = M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision=prec)
        s = np.zeros((w.n_rve, 6))
        assert g.run(w.F, s, update_coords=False)
        out[prec] = s
    err = np.abs(out["mixed"] - out["f64"]).max(axis=1) / np.abs(out["f64"]).max(axis=1)
    assert err.max() <= REL_MIXED, err


def test_config2_largest_rves_mixed_vs_fp64(M, config2_large):
    """Config 2's largest RVEs at its 5,000 steps: mixed within 1e-5 of FP64
    (these RVEs are solved by 4-CTA clusters)."""
    from mumfim_gb300 import synthetic as S
    w = config2_large
    w = S.Workload(w.name, w.networks, [M.SolutionStrategy.ramp(5_000, 0.5)] * w.n_rve, w.F,
                   5_000)
    out = {}
    for prec in ("f64", "mixed"):
        g = M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision=prec)
        s = np.zeros((w.n_rve, 6))
        assert g.run(w.F, s, update_coords=False)
        out[prec] = s
    err = np.abs(out["mixed"] - out["f64"]).max(axis=1) / np.abs(out["f64"]).max(axis=1)
    assert err.max() <= REL_MIXED, err
