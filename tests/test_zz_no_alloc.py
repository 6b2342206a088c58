"""The solve for callers that cannot allocate device memory.

Some callers of this library must not allocate device memory while they
solve. One example is a macroscale code whose GPU memory is owned by its own
pool allocator. Another is a time-stepping loop that forbids allocation after
start-up. mfg_batch_run_device_noalloc() serves them. It runs the FP64
relaxation with its scratch taken from a fixed device array inside the
library instead of buffers allocated with the batch.

These tests call it through the C ABI and compare it with the allocating
mfg_batch_run_device() on identical batches. The FP64 kernel is bit-exact, so
the tolerance is the one the other FP64 tests use: equality. Two updating
calls run in a row, so the second one also sees the fixed array as the first
call left it. This file is collected last, and it passes whether it runs
alone in a fresh process or after the other tests.
"""
import numpy as np
import pytest

from conftest import network_2_7

pytestmark = pytest.mark.gpu


def _batches(m, S, n_rve, n_nodes, steps):
    w = S.config1(n_rve=n_rve, n_nodes=n_nodes, steps=steps)
    return (w, m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies),
            m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies))


def test_noalloc_solve_matches_allocating_solve_twice_in_a_row(lib_path):
    import torch

    import mumfim_gb300 as m
    from mumfim_gb300 import synthetic as S

    R = 4
    w, alloc, noalloc = _batches(m, S, R, 800, 600)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    with torch.cuda.stream(stream):
        F1 = torch.from_numpy(np.ascontiguousarray(w.F.reshape(R, 9))).to(dev)
        shear = np.eye(3) + 0.02 * np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]])
        F2 = torch.from_numpy(np.ascontiguousarray(np.repeat(shear.reshape(1, 9), R, 0))).to(dev)
    stream.synchronize()
    for F in (F1, F2):
        with torch.cuda.stream(stream):
            s_a = torch.zeros((R, 6), dtype=torch.float64, device=dev)
            s_n = torch.full((R, 6), float("nan"), dtype=torch.float64, device=dev)
            st_a = torch.zeros((R, 2), dtype=torch.float64, device=dev)
            st_n = torch.zeros((R, 2), dtype=torch.float64, device=dev)
        stream.synchronize()
        alloc.run_device(F.data_ptr(), R, s_a.data_ptr(), True, st_a.data_ptr(), stream.cuda_stream)
        noalloc.run_device_noalloc(F.data_ptr(), R, s_n.data_ptr(), True, st_n.data_ptr(),
                                   stream.cuda_stream)
        stream.synchronize()
        assert torch.equal(s_a, s_n)
        assert torch.equal(st_a, st_n)
        assert bool(torch.isfinite(s_n).all())
    for r in range(R):
        np.testing.assert_array_equal(alloc.displacements(r), noalloc.displacements(r))
    np.testing.assert_array_equal(alloc.current_stress(), noalloc.current_stress())


def test_noalloc_relax_mode_and_non_updating_run(lib_path, golden_2_7):
    """RELAX mode (the reference's algorithm): RVEs that converge and one
    stopped by its step cap (status MFG_E_NOT_CONVERGED), an updating run,
    then a non-updating run with one broadcast F and no status output. The
    non-updating run must leave u and the stored stress as they were, in both
    paths, bit for bit."""
    import torch

    import mumfim_gb300 as m
    from mumfim_gb300 import synthetic as S

    R = 3
    # Network_2_7 with its damping converges (in about 20,600 steps); the
    # third RVE is stopped by its step cap
    net = network_2_7(golden_2_7)
    w = S.config1(n_rve=1, n_nodes=600)
    nets = [net, net, w.networks[0]]
    strat = [m.SolutionStrategy(visc_damp_coeff=golden_2_7["visc_damp_coeff"], residual_tol=1e-6,
                                max_steps=40_000)] * 2 + [
        m.SolutionStrategy(visc_damp_coeff=0.5, residual_tol=1e-30, max_steps=250)]
    alloc = m.BatchedFiberRVEAnalysisExplicit(nets, strat)
    noalloc = m.BatchedFiberRVEAnalysisExplicit(nets, strat)
    F_gold = np.array(golden_2_7["F"]).reshape(3, 3)
    F_all = np.stack([F_gold, F_gold.T, w.F[0]])
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    with torch.cuda.stream(stream):
        F1 = torch.from_numpy(np.ascontiguousarray(F_all.reshape(R, 9))).to(dev)
        tilt = np.eye(3) + 0.01 * np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, -1.0]])
        F2 = torch.from_numpy(np.ascontiguousarray(tilt.reshape(1, 9))).to(dev)
        st_a = torch.zeros((R, 2), dtype=torch.float64, device=dev)
        st_n = torch.zeros((R, 2), dtype=torch.float64, device=dev)
        s_a = torch.zeros((R, 6), dtype=torch.float64, device=dev)
        s_n = torch.full((R, 6), float("nan"), dtype=torch.float64, device=dev)
    stream.synchronize()
    alloc.run_device(F1.data_ptr(), R, s_a.data_ptr(), True, st_a.data_ptr(), stream.cuda_stream)
    noalloc.run_device_noalloc(F1.data_ptr(), R, s_n.data_ptr(), True, st_n.data_ptr(),
                               stream.cuda_stream)
    stream.synchronize()
    assert torch.equal(s_a, s_n)
    assert torch.equal(st_a, st_n)
    status = st_n.cpu().numpy().view(m.RVE_STATUS_DTYPE).reshape(R)
    assert list(status["status"]) == [0, 0, 3]
    assert status["steps"][2] == 250
    u_before = [noalloc.displacements(r) for r in range(R)]
    cur_before = noalloc.current_stress()
    with torch.cuda.stream(stream):
        s_a2 = torch.zeros((R, 6), dtype=torch.float64, device=dev)
        s_n2 = torch.full((R, 6), float("nan"), dtype=torch.float64, device=dev)
    stream.synchronize()
    alloc.run_device(F2.data_ptr(), 1, s_a2.data_ptr(), False, 0, stream.cuda_stream)
    noalloc.run_device_noalloc(F2.data_ptr(), 1, s_n2.data_ptr(), False, 0, stream.cuda_stream)
    stream.synchronize()
    assert torch.equal(s_a2, s_n2)
    assert bool(torch.isfinite(s_n2).all())
    for r in range(R):
        np.testing.assert_array_equal(noalloc.displacements(r), u_before[r])
        np.testing.assert_array_equal(alloc.displacements(r), u_before[r])
        np.testing.assert_array_equal(alloc.displacements(r), noalloc.displacements(r))
        np.testing.assert_array_equal(alloc.coordinates(r), noalloc.coordinates(r))
    np.testing.assert_array_equal(noalloc.current_stress(), cur_before)
    np.testing.assert_array_equal(alloc.current_stress(), noalloc.current_stress())


_FRESH = r"""
import json, sys
import numpy as np
import torch
sys.path.insert(0, {repo!r})
import mumfim_gb300 as m
from mumfim_gb300 import synthetic as S
R = 3
w = S.config1(n_rve=R, n_nodes=700, steps=500)
dev = torch.device("cuda", 0)
F = torch.from_numpy(np.ascontiguousarray(w.F.reshape(R, 9))).to(dev)
s_n = torch.zeros((R, 6), dtype=torch.float64, device=dev)
s_a = torch.zeros((R, 6), dtype=torch.float64, device=dev)
noalloc = m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies)
torch.cuda.synchronize(dev)
free0 = torch.cuda.mem_get_info(dev)[0]
noalloc.run_device_noalloc(F.data_ptr(), R, s_n.data_ptr(), True)
torch.cuda.synchronize(dev)
free1 = torch.cuda.mem_get_info(dev)[0]
alloc = m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies)
alloc.run_device(F.data_ptr(), R, s_a.data_ptr(), True)
torch.cuda.synchronize(dev)
print(json.dumps({{"drop": int(free0 - free1), "equal": bool(torch.equal(s_a, s_n)),
                  "finite": bool(torch.isfinite(s_n).all())}}))
"""


def test_noalloc_first_solve_of_a_fresh_process(lib_path):
    """The first solve a process makes is the no-allocation one: device
    memory must not shrink by the fixed array's size during it (batch
    creation has already reserved the array), and its result must equal the
    allocating solve's."""
    import json
    import os
    import subprocess
    import sys

    import mumfim_gb300 as m

    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "-c", _FRESH.format(repo=repo)], capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    res = json.loads(out.stdout.strip().splitlines()[-1])
    assert res["equal"] and res["finite"]
    assert res["drop"] < m.NOALLOC_SCRATCH_BYTES, res


def test_noalloc_solve_rejects_batches_beyond_the_fixed_array(lib_path):
    import torch

    import mumfim_gb300 as m
    from mumfim_gb300 import synthetic as S

    # 48 RVEs x 4500 nodes need about 18 MB of scratch, above the 16 MiB array.
    R = 48
    w = S.config1(n_rve=R, n_nodes=4500, steps=10)
    big = m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies)
    dev = torch.device("cuda", 0)
    F = torch.from_numpy(np.ascontiguousarray(w.F.reshape(R, 9))).to(dev)
    s = torch.zeros((R, 6), dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    with pytest.raises(m.MumfimGpuError) as ei:
        big.run_device_noalloc(F.data_ptr(), R, s.data_ptr(), True)
    assert ei.value.status == 1
    assert "bytes of scratch" in str(ei.value)
