"""Launch-shape autotuner: it times candidate shapes (largest cluster,
serving layout, solve of small RVEs) on a size-stratified sample of the batch,
picks the fastest and caches the choice per GPU and size mix; a shape changes
speed, never results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tune_launch_shape_and_cache(lib_path, tmp_path, monkeypatch):
    import mumfim_gb300 as m
    from mumfim_gb300 import synthetic as S
    from mumfim_gb300.autotune import LaunchShape, tune_launch_shape
    monkeypatch.setenv("MFG_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    w = S.config2(n_rve=24, steps=200, n_min=600, n_max=14_000)
    cands = [LaunchShape(8, False, 0, "node"), LaunchShape(4, True, 1, "fiber"),
             LaunchShape(1, False, 2, "fiber")]
    best, rep = tune_launch_shape(w.networks, w.strategies, w.F, steps=40, sample=16,
                                  repeats=1, candidates=cands)
    assert not rep["from_cache"] and rep["sample_rves"] == 16
    rates = [t["fiber_steps_per_s"] for t in rep["table"]]
    assert len(rates) == 3 and all(r > 0 for r in rates)
    assert best == LaunchShape(**rep["table"][int(np.argmax(rates))]["shape"])
    again, rep2 = tune_launch_shape(w.networks, w.strategies, w.F, steps=40, sample=16,
                                    repeats=1, candidates=cands)
    assert rep2["from_cache"] and again == best
    sig = []
    for shape in (best, *cands):
        g = m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision="mixed",
                                              **shape.kwargs())
        s = np.zeros((w.n_rve, 6))
        g.run(w.F, s, update_coords=False)
        sig.append(s)
        g.close()
    for s in sig[1:]:
        np.testing.assert_array_equal(sig[0], s)


def test_tune_cluster_limit(lib_path):
    from mumfim_gb300 import synthetic as S
    from mumfim_gb300.autotune import tune_cluster_limit
    w = S.config2(n_rve=16, steps=200, n_min=2_000, n_max=14_000)
    best, table = tune_cluster_limit(w.networks, w.strategies, w.F, steps=40,
                                     candidates=(1, 4), repeats=1)
    assert set(table) == {1, 4} and best in table
    assert all(v > 0 for v in table.values()) and table[best] == max(table.values())
