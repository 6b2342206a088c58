"""Launch-shape autotuner: it times every candidate cluster-size limit on
the batch and picks the fastest; the limit changes speed, not results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tune_cluster_limit(lib_path):
    import mumfim_gb300 as m
    from mumfim_gb300 import synthetic as S
    from mumfim_gb300.autotune import tune_cluster_limit
    w = S.config2(n_rve=16, steps=200, n_min=2_000, n_max=14_000)
    best, table = tune_cluster_limit(w.networks, w.strategies, w.F, steps=40,
                                     candidates=(1, 4), repeats=1)
    assert set(table) == {1, 4} and best in table
    assert all(v > 0 for v in table.values()) and table[best] == max(table.values())
    sig = []
    for limit in (best, 0):
        g = m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision="mixed",
                                              max_cluster_ctas=limit)
        s = np.zeros((w.n_rve, 6))
        g.run(w.F, s, update_coords=False)
        sig.append(s)
        g.close()
    np.testing.assert_array_equal(sig[0], sig[1])
