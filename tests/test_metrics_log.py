"""The structured metrics sink: one JSON object per line for each C-ABI
call, failures included (status and message), so a service loop can log
what every run did."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import REPO


def _records(path):
    with open(path) as fh:
        return [json.loads(line) for line in fh if line.strip()]


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_failed_calls_are_recorded(lib_path, tmp_path):
    import mumfim_gb300 as m
    from mumfim_gb300 import synthetic as S
    from mumfim_gb300.batched import set_metrics_log
    log = tmp_path / "metrics.jsonl"
    set_metrics_log(str(log))
    try:
        w = S.config1(n_rve=2, n_nodes=300, steps=50)
        with pytest.raises(m.MumfimGpuError):
            m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision="mixed",
                                              max_cluster_ctas=3)
        if not _has_gpu():
            with pytest.raises(m.MumfimGpuError):
                m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies)
    finally:
        set_metrics_log(None)
    rec = _records(log)
    assert rec[0]["call"] == "mfg_batch_create" and rec[0]["status"] == "MFG_E_INVALID"
    assert "max_cluster_ctas" in rec[0]["message"] and rec[0]["n_rve"] == 2
    if not _has_gpu():
        assert rec[1]["status"] == "MFG_E_NO_DEVICE"
    assert all(isinstance(r["t"], float) for r in rec)


def test_environment_variable_turns_it_on(lib_path, tmp_path):
    log = tmp_path / "env.jsonl"
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import mumfim_gb300 as m\nfrom mumfim_gb300 import synthetic as S\n"
            "w = S.config1(n_rve=1, n_nodes=300, steps=50)\n"
            "try:\n    m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision='x')\n"
            "except Exception:\n    pass\n"
            "try:\n    m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, small_rves_per_cta=5)\n"
            "except Exception:\n    pass\n") % REPO
    env = dict(os.environ, MFG_METRICS_LOG=str(log))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    rec = _records(log)
    assert len(rec) == 1 and rec[0]["status"] == "MFG_E_INVALID"
    assert "small_rves_per_cta" in rec[0]["message"]


@pytest.mark.gpu
def test_run_stiffness_and_server_records(lib_path, tmp_path):
    import mumfim_gb300 as m
    from mumfim_gb300 import synthetic as S
    from mumfim_gb300.batched import set_metrics_log
    from mumfim_gb300.serving import RVEServer
    log = tmp_path / "metrics.jsonl"
    w = S.config2(n_rve=6, steps=300, n_min=500, n_max=6000)
    set_metrics_log(str(log))
    try:
        g = m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision="mixed")
        g.run(w.F, update_coords=True)
        g.computeMaterialStiffness()
        g.close()
        with RVEServer(w.networks, w.strategies) as sv:
            for r in range(w.n_rve):
                sv.submit(r, w.F[r], update_coords=False)
            sv.drain()
    finally:
        set_metrics_log(None)
    rec = _records(log)
    calls = [r["call"] for r in rec]
    assert calls[:3] == ["mfg_batch_create", "mfg_batch_run", "mfg_batch_material_stiffness"]
    run = rec[1]
    assert run["status"] == "MFG_OK" and run["ok"] == w.n_rve and run["n_rve"] == w.n_rve
    assert run["steps_min"] == run["steps_max"] == 300
    assert run["fiber_steps"] == pytest.approx(w.total_fibers * 300)
    assert run["relax_ms"] > 0 and run["run_ms"] >= run["relax_ms"]
    assert rec[2]["solves"] == "concurrent"  # one record: the six inner solves are not logged
    polls = [r for r in rec if r["call"] == "mfg_server_poll"]
    assert sum(p["results"] for p in polls) == w.n_rve
    assert all(p["latency_ms_max"] >= p["latency_ms_mean"] > 0 for p in polls)
