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
