"""Mixed-precision kernel (FP32 forces and integrator, FP64 reference
coordinates + Kahan-compensated FP32 displacements, FP64 stress / residual /
dt) against the plain FP64 kernel and the oracle.

Tolerance: 1e-5 relative stress error against FP64 (the target the mixed
path is specified to), measured as max |sigma_mixed - sigma_f64| over the
largest |sigma_f64| of the batch.
"""
import numpy as np
import pytest

from conftest import network_2_7, voigt_to_mat

pytestmark = pytest.mark.gpu

REL_MIXED = 1e-5


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.fixture(scope="module")
def M(lib_path):
    import mumfim_gb300 as m
    return m


def _solve(M, w, precision, opts=None, **kw):
    g = M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision=precision,
                                          **(opts or {}))
    sig = np.zeros((w.n_rve, 6))
    g.run(w.F, sig, **kw)
    return g, sig


def test_mixed_config1_subset_within_1e5_of_f64(M):
    from mumfim_gb300 import synthetic as S
    w = S.config1(n_rve=16, steps=5_000)
    g64, s64 = _solve(M, w, "f64")
    g32, s32 = _solve(M, w, "mixed")
    assert (g32.last_status["steps"] == 5_000).all()
    assert _rel(s32, s64) <= REL_MIXED
    for r in (0, 9):
        assert _rel(g32.displacements(r), g64.displacements(r)) <= REL_MIXED


def test_mixed_config2_uneven_subset(M):
    from mumfim_gb300 import synthetic as S
    w = S.config2(n_rve=12, steps=2_000)
    g64, s64 = _solve(M, w, "f64")
    g32, s32 = _solve(M, w, "mixed")
    assert _rel(s32, s64) <= REL_MIXED


def test_mixed_nonlinear_law(M, oracle):
    from mumfim_gb300 import synthetic as S
    w = S.config3(n_rve=6, steps=3_000, n_min=500, n_max=1200)
    g64, s64 = _solve(M, w, "f64")
    g32, s32 = _solve(M, w, "mixed")
    assert _rel(s32, s64) <= REL_MIXED


def test_mixed_relax_network_2_7(M, golden_2_7):
    g = golden_2_7
    net = network_2_7(g)
    s = M.SolutionStrategy(visc_damp_coeff=g["visc_damp_coeff"], residual_tol=1e-6)
    gpu = M.BatchedFiberRVEAnalysisExplicit([net], [s], precision="mixed")
    F = np.array(g["F"]).reshape(1, 3, 3)
    sig = np.zeros((1, 6))
    assert gpu.run(F, sig)
    assert gpu.last_status["steps"][0] % 100 == 1
    gold = np.array(g["outputs"]["explicit_cpu_out"]["stress"][0])
    J = np.linalg.det(F[0])
    assert np.abs(voigt_to_mat(sig[0] * J) - gold).max() <= 1e-5 * np.abs(gold).max()


def test_mixed_incremental_and_transactional_runs(M):
    from mumfim_gb300 import synthetic as S
    w = S.config1(n_rve=3, n_nodes=700, steps=1_500)
    a = M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision="f64")
    b = M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision="mixed")
    F2 = np.repeat((np.eye(3) + 0.01 * np.array([[0, 1, 0], [0, 0, 0], [0, 0, -1.0]]))[None], 3, 0)
    for F, upd in ((w.F, True), (F2, True), (F2[:1], False), (w.F, True)):
        sa, sb = np.zeros((3, 6)), np.zeros((3, 6))
        a.run(F, sa, update_coords=upd)
        b.run(F, sb, update_coords=upd)
        assert _rel(sb, sa) <= REL_MIXED
    for r in range(3):
        assert _rel(b.displacements(r), a.displacements(r)) <= REL_MIXED
    np.testing.assert_allclose(b.compute3DOrientationTensor(), a.compute3DOrientationTensor(),
                               rtol=0, atol=1e-9)


def test_mixed_every_placement_and_cluster_size(M):
    """One RVE per way a batch run places an RVE: node-centric with two
    copies of the node records on one CTA (800 nodes) and over clusters of
    2 and 4 CTAs (7,000 / 14,000), with one copy on one CTA (4,000) and over
    clusters of 2, 4 and 8 CTAs (9,000 / 20,000 / 40,000), fiber-centric in
    global memory (80,000), and on
    request fiber-centric with all mutable state in one CTA's shared memory
    (800, 4,000). Each agrees with FP64, and each gives the same bits solved
    alone as in the mixed-size batch, whichever solve."""
    from mumfim_gb300 import synthetic as S
    sizes = (800, 4_000, 9_000, 20_000, 40_000, 80_000, 7_000, 14_000)
    nets, F = [], []
    for i, n in enumerate(sizes):
        coords, conn = S.knn_network(n, 4, S.geometry_seed(7, i))
        nets.append(M.FiberNetwork(coords, conn, [S._linear_params(7, i)]))
        u = S.uniform(S.param_seed(7, i), 9) * 0.1 - 0.05
        F.append(np.eye(3) + u.reshape(3, 3))
    strat = [M.SolutionStrategy.ramp(1_000, 0.5) for _ in nets]
    F = np.stack(F)
    w = S.Workload("placements", nets, strat, F, 1_000)
    g64, s64 = _solve(M, w, "f64")
    g32, s32 = _solve(M, w, "mixed")
    assert (g32.last_status["steps"] == 1_000).all()
    # one launch per non-empty size bucket -- node-centric with two record
    # copies on 1, 2 and 4 CTAs, with one on 1, 2, 4 and 8 CTAs, the
    # run-time placement -- and the status pack
    assert g32.last_launches() == 8 + 1
    for r in range(len(sizes)):
        assert _rel(s32[r], s64[r]) <= REL_MIXED, r
    for r in (0, 2, 4, 5, 6, 7):
        one = w.subset([r])
        _, s1 = _solve(M, one, "mixed")
        np.testing.assert_array_equal(s1[0], s32[r])
    gf, sf = _solve(M, w.subset([0, 1]), "mixed", {"small_rve_solve": "fiber"})
    assert gf.last_launches() == 2 + 1  # fiber-centric pair (800), node-centric (4,000)
    np.testing.assert_array_equal(sf, s32[:2])


def test_cluster_and_single_cta_solves_agree(M):
    """The same RVEs solved node-centric over thread-block clusters (1, 2, 4
    and 8 CTAs, with one or two copies of the node records), in the serving
    layout (clusters of 4 instead of 2) and on
    one CTA each (max_cluster_ctas=1: node-centric where the node state
    fits, else fiber-centric with run-time placement): the same per-fiber
    and per-node arithmetic in the same order, so the same bits, in RAMP
    mode and in RELAX mode (there the step count too; only the residual's
    last bits may differ, since a cluster sums it in per-CTA parts)."""
    from mumfim_gb300 import synthetic as S
    sizes = (4_000, 9_000, 20_000, 40_000, 7_000, 14_000)
    nets, F = [], []
    for i, n in enumerate(sizes):
        coords, conn = S.knn_network(n, 4, S.geometry_seed(11, i))
        nets.append(M.FiberNetwork(coords, conn, [S._linear_params(11, i)]))
        F.append(np.eye(3) + (S.uniform(S.param_seed(11, i), 9) * 0.06 - 0.03).reshape(3, 3))
    F = np.stack(F)
    for strat in (M.SolutionStrategy.ramp(800, 0.5),
                  M.SolutionStrategy(visc_damp_coeff=0.5, residual_tol=1e-6, max_steps=1_500)):
        out = []
        for mc, sl in ((0, False), (1, False), (0, True)):
            g = M.BatchedFiberRVEAnalysisExplicit(nets, [strat] * len(nets), precision="mixed",
                                                  max_cluster_ctas=mc, serving_layout=sl)
            s = np.zeros((len(nets), 6))
            g.run(F, s)
            out.append((s, g.last_status.copy(), g.displacements(2)))
            g.close()
        s0, st0, u0 = out[0]
        for s1, st1, u1 in out[1:]:
            np.testing.assert_array_equal(s0, s1)
            np.testing.assert_array_equal(u0, u1)
            np.testing.assert_array_equal(st0["steps"], st1["steps"])
            np.testing.assert_array_equal(st0["status"], st1["status"])
            np.testing.assert_allclose(st0["residual"], st1["residual"], rtol=1e-9)


def test_max_cluster_ctas_is_checked(M):
    from mumfim_gb300 import synthetic as S
    w = S.config1(n_rve=1, n_nodes=300, steps=10)
    with pytest.raises(M.MumfimGpuError, match="max_cluster_ctas"):
        M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision="mixed",
                                          max_cluster_ctas=3)


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_degenerate_networks_match_oracle(M, oracle, precision):
    """Networks at the edges of the set-up: every node on the boundary (no
    free node: the solve only moves the boundary), no boundary node (the
    RAMP increments move nothing), and a two-node, one-fiber RVE. FP64 is
    bit-identical to the oracle; mixed agrees within 1e-5 of the largest
    stress component (or 1e-12 absolute when the stress is zero)."""
    from mumfim_gb300.network_io import FiberNetwork, Reaction
    r = [Reaction(0, 1e-3, 1.0, 1.0)]
    all_bnd = FiberNetwork(np.array([[-0.5, -0.5, 0.1], [0.5, -0.2, 0.3], [0.1, 0.5, -0.5],
                                     [-0.2, 0.3, 0.5]]),
                           np.array([[0, 1], [1, 2], [2, 3], [3, 0], [0, 2]], dtype=np.int32), r)
    no_bnd = FiberNetwork(np.array([[0.0, 0.0, 0.0], [0.2, 0.0, 0.0], [0.1, 0.15, 0.0],
                                    [0.1, 0.05, 0.2]]),
                          np.array([[0, 1], [1, 2], [2, 0], [0, 3], [1, 3], [2, 3]],
                                   dtype=np.int32), r)
    pair = FiberNetwork(np.array([[-0.5, 0.0, 0.0], [0.5, 0.1, 0.0]]),
                        np.array([[0, 1]], dtype=np.int32), r)
    nets = [all_bnd, no_bnd, pair]
    strat = [M.SolutionStrategy.ramp(50, 0.5) for _ in nets]
    F = np.repeat((np.eye(3) + 0.02 * np.array([[1.0, 0.3, 0], [0, -0.5, 0], [0.1, 0, 0.2]]))[None],
                  3, 0)
    g = M.BatchedFiberRVEAnalysisExplicit(nets, strat, precision=precision)
    s = np.zeros((3, 6))
    g.run(F, s)
    rc, so, _ = oracle.OracleBatch(nets, strat).run(F)
    assert (g.last_status["status"] == 0).all()
    if precision == "f64":
        np.testing.assert_array_equal(s, so)
    else:
        for k in range(3):
            scale = np.abs(so[k]).max()
            assert np.abs(s[k] - so[k]).max() <= max(1e-5 * scale, 1e-12), (k, s[k], so[k])


def test_graph_replay_and_recapture(M):
    """A mixed batch run is a CUDA graph captured for its arguments and
    replayed while they stay the same: repeated non-updating runs give the
    same bits, and a run with other device buffers (a recapture) gives them
    too."""
    import torch
    from mumfim_gb300 import synthetic as S
    w = S.config2(n_rve=24, steps=300, n_min=500, n_max=14_000)
    g = M.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision="mixed")
    outs = []
    for _ in range(3):
        s = np.zeros((w.n_rve, 6))
        g.run(w.F, s, update_coords=False)
        outs.append(s)
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])
    for _ in range(2):
        F_dev = torch.tensor(w.F.reshape(-1, 9), dtype=torch.float64, device="cuda")
        sig_dev = torch.zeros((w.n_rve, 6), dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream()
        g.run_device(F_dev.data_ptr(), w.n_rve, sig_dev.data_ptr(), update_coords=False,
                     stream=stream.cuda_stream)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(sig_dev.cpu().numpy(), outs[0])


def test_paired_small_rves_match_one_per_cta(M):
    """With the fiber-centric small solve, small RVEs (whole state within
    half a CTA's shared memory) are solved two per CTA, each by a 512-thread
    group with its own named barrier; the group reductions keep the order of
    a whole CTA, so the stresses, displacements, step counts and statuses
    are those of one RVE per CTA, and those of the node-centric solve, in
    RAMP and in RELAX mode."""
    from mumfim_gb300 import synthetic as S
    w = S.config2(n_rve=24, steps=700, n_min=500, n_max=2_500)
    for strat in (w.strategies,
                  [M.SolutionStrategy(visc_damp_coeff=2.0, residual_tol=1e-7, max_steps=2_000)]
                  * w.n_rve):
        out = []
        for solve, per_cta in (("fiber", 2), ("fiber", 1), ("node", 0)):
            g = M.BatchedFiberRVEAnalysisExplicit(w.networks, strat, precision="mixed",
                                                  small_rve_solve=solve,
                                                  small_rves_per_cta=per_cta)
            s = np.zeros((w.n_rve, 6))
            g.run(w.F, s)
            out.append((s, g.last_status.copy(), [g.displacements(r) for r in (0, 5, 23)]))
            g.close()
        s2, st2, u2 = out[0]
        for k, (s1, st1, u1) in enumerate(out[1:]):
            np.testing.assert_array_equal(s2, s1)
            np.testing.assert_array_equal(st2["steps"], st1["steps"])
            np.testing.assert_array_equal(st2["status"], st1["status"])
            if k == 0:  # the pair's group sums keep a whole CTA's order
                np.testing.assert_array_equal(st2["residual"], st1["residual"])
            else:  # the node-centric order sums the residual in another order
                np.testing.assert_allclose(st2["residual"], st1["residual"], rtol=1e-9)
            for a, b in zip(u2, u1):
                np.testing.assert_array_equal(a, b)
