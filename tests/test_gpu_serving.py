"""Continuous-batching server: requests join the running persistent kernel,
results equal the batch API's, and a result does not depend on what else is
in flight (deterministic per-RVE solves: bit-identical alone and in the mix)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def W(lib_path):
    from mumfim_gb300 import synthetic as S
    return S.config2(n_rve=10, steps=800, n_min=400, n_max=3000)


def _batch_sigma(m, w, precision, F=None, update=False):
    g = m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision=precision)
    sig = np.zeros((w.n_rve, 6))
    g.run(w.F if F is None else F, sig, update_coords=update)
    return sig


@pytest.mark.parametrize("precision", ["mixed", "f64"])
def test_alone_equals_in_the_mix_equals_batch(W, precision):
    import mumfim_gb300 as m
    from mumfim_gb300.serving import RVEServer
    ref = _batch_sigma(m, W, precision)
    with RVEServer(W.networks, W.strategies, precision=precision) as sv:
        sv.submit(3, W.F[3], update_coords=False)
        alone = sv.drain()
        assert len(alone) == 1 and alone["rve"][0] == 3
        for r in range(W.n_rve):
            sv.submit(r, W.F[r], update_coords=False)
        mix = sv.drain()
    assert sorted(mix["rve"].tolist()) == list(range(W.n_rve))
    np.testing.assert_array_equal(alone["sigma"][0], mix["sigma"][mix["rve"] == 3][0])
    for rec in mix:
        np.testing.assert_array_equal(rec["sigma"], ref[rec["rve"]])
        assert rec["status"] == 0 and rec["steps"] == 800


def test_requests_join_while_others_run(W):
    """Submissions spread over time: later requests are claimed by CTAs
    while earlier solves are still on the device (continuous batching)."""
    import mumfim_gb300 as m
    from mumfim_gb300.serving import RVEServer
    ref = _batch_sigma(m, W, "mixed")
    got = []
    with RVEServer(W.networks, W.strategies, precision="mixed") as sv:
        for r in range(W.n_rve):
            sv.submit(r, W.F[r], update_coords=False)
            time.sleep(0.002)
            got.append(sv.poll(timeout_ms=0))
        got.append(sv.drain())
    res = np.concatenate(got)
    assert len(res) == W.n_rve
    for rec in res:
        np.testing.assert_array_equal(rec["sigma"], ref[rec["rve"]])
    # some request was claimed before an earlier-claimed one finished
    order = np.argsort(res["t_claim_ns"])
    claims, dones = res["t_claim_ns"][order], res["t_done_ns"][order]
    assert any(claims[i + 1] < dones[i] for i in range(len(order) - 1))
    assert (res["latency_s"] >= res["device_s"]).all()


def test_same_rve_requests_run_in_submission_order(W):
    """Two updating increments on one RVE: the second waits for the first and
    the final state equals two sequential batch runs."""
    import mumfim_gb300 as m
    from mumfim_gb300.serving import RVEServer
    F2 = np.eye(3) + 0.01 * np.array([[0, 1.0, 0], [0, 0, 0], [0, 0, -0.5]])
    g = m.BatchedFiberRVEAnalysisExplicit(W.networks, W.strategies, precision="mixed")
    s1, s2 = np.zeros((W.n_rve, 6)), np.zeros((W.n_rve, 6))
    g.run(W.F, s1, update_coords=True)
    g.run(np.repeat(F2[None], W.n_rve, 0), s2, update_coords=True)
    with RVEServer(W.networks, W.strategies, precision="mixed") as sv:
        t1 = sv.submit(5, W.F[5], update_coords=True)
        t2 = sv.submit(5, F2, update_coords=True)
        res = sv.drain()
    res = res[np.argsort(res["ticket"])]
    assert res["ticket"].tolist() == [t1, t2]
    np.testing.assert_array_equal(res["sigma"][0], s1[5])
    np.testing.assert_array_equal(res["sigma"][1], s2[5])


def test_admission_ring_full_and_idle_relaunch(W):
    import mumfim_gb300 as m
    from mumfim_gb300.serving import RVEServer
    with pytest.raises(m.MumfimGpuError) as ei:
        RVEServer(W.networks, W.strategies, hbm_budget_bytes=1e5)
    assert ei.value.status == 8 and "admission refused" in str(ei.value)
    with RVEServer(W.networks, W.strategies, capacity=4, idle_timeout_us=1000) as sv:
        for r in range(4):
            sv.submit(r, W.F[r], update_coords=False)
        with pytest.raises(m.MumfimGpuError) as ei:
            sv.submit(4, W.F[4], update_coords=False)
        assert ei.value.status == 8
        assert len(sv.drain()) == 4
        time.sleep(0.05)  # the kernel leaves after 1 ms without work
        sv.submit(6, W.F[6], update_coords=False)
        assert len(sv.drain()) == 1
        assert sv.launches() >= 2


def test_server_placements_match_clustered_batch(lib_path):
    """The serving kernel solves each RVE with the solve of its bucket in the
    serving layout: fiber-centric on one CTA (1,000 nodes), node-centric on
    one CTA (5,000) and node-centric over clusters of 4 (8,000 and 12,000),
    while a batch run takes a cluster of 2 for 8,000: the ramped stress is
    the same bits either way (same per-fiber and per-node arithmetic, and dt
    is a minimum)."""
    import mumfim_gb300 as m
    from mumfim_gb300 import synthetic as S
    from mumfim_gb300.serving import RVEServer
    sizes = (1_000, 5_000, 8_000, 12_000)
    nets, F = [], []
    for i, n in enumerate(sizes):
        coords, conn = S.knn_network(n, 4, S.geometry_seed(8, i))
        nets.append(m.FiberNetwork(coords, conn, [S._linear_params(8, i)]))
        F.append(np.eye(3) + (S.uniform(S.param_seed(8, i), 9) * 0.1 - 0.05).reshape(3, 3))
    w = S.Workload("server placements", nets, [m.SolutionStrategy.ramp(600, 0.5) for _ in nets],
                   np.stack(F), 600)
    ref = _batch_sigma(m, w, "mixed")
    with RVEServer(w.networks, w.strategies, precision="mixed") as sv:
        for r in range(w.n_rve):
            sv.submit(r, w.F[r], update_coords=False)
        res = sv.drain()
    assert len(res) == w.n_rve
    for rec in res:
        assert rec["status"] == 0
        np.testing.assert_array_equal(rec["sigma"], ref[rec["rve"]])


def test_cluster_lane_holds_requests_per_rve(lib_path):
    """Two updating increments on an RVE the server solves with a cluster
    (8,000 nodes) and on a small one, interleaved: each RVE's second request
    waits for its first, and both end states equal two sequential batch
    runs."""
    import mumfim_gb300 as m
    from mumfim_gb300 import synthetic as S
    from mumfim_gb300.serving import RVEServer
    nets = []
    for i, n in enumerate((8_000, 1_200)):
        coords, conn = S.knn_network(n, 4, S.geometry_seed(10, i))
        nets.append(m.FiberNetwork(coords, conn, [S._linear_params(10, i)]))
    strat = [m.SolutionStrategy.ramp(400, 0.5) for _ in nets]
    F1 = np.eye(3) + 0.01 * np.array([[0, 1.0, 0], [0, 0, 0], [0, 0, -0.5]])
    F2 = np.eye(3) + 0.01 * np.array([[0.5, 0, 0], [0, -0.2, 0.1], [0, 0, 0]])
    g = m.BatchedFiberRVEAnalysisExplicit(nets, strat, precision="mixed")
    s1, s2 = np.zeros((2, 6)), np.zeros((2, 6))
    g.run(np.stack([F1, F1]), s1, update_coords=True)
    g.run(np.stack([F2, F2]), s2, update_coords=True)
    with RVEServer(nets, strat, precision="mixed") as sv:
        t = [sv.submit(0, F1), sv.submit(1, F1), sv.submit(0, F2), sv.submit(1, F2)]
        res = sv.drain()
    assert len(res) == 4
    by_ticket = {int(r["ticket"]): r for r in res}
    for rve, (a, b) in enumerate(((t[0], t[2]), (t[1], t[3]))):
        np.testing.assert_array_equal(by_ticket[a]["sigma"], s1[rve])
        np.testing.assert_array_equal(by_ticket[b]["sigma"], s2[rve])
        assert by_ticket[b]["t_claim_ns"] >= by_ticket[a]["t_done_ns"]


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_served_stiffness_equals_batch_run_then_stiffness(lib_path, precision):
    """A request with stiffness=True returns a full micro_fo_result: the
    stress of its (updating) solve and the material stiffness of the six
    perturbed solves that follow it on the same CTA or cluster, bit-identical
    to mfg_batch_run followed by a sequential mfg_batch_material_stiffness.
    RVEs of 1,000 - 9,000 nodes: the mixed server solves the largest with
    4-CTA clusters. A request without the flag reports stiffness_status -1."""
    import mumfim_gb300 as m
    from mumfim_gb300 import synthetic as S
    from mumfim_gb300.serving import RVEServer
    w = S.config2(n_rve=6, steps=500, n_min=1_000, n_max=9_000)
    g = m.BatchedFiberRVEAnalysisExplicit(w.networks, w.strategies, precision=precision,
                                          stiffness="sequential")
    s_ref = np.zeros((w.n_rve, 6))
    g.run(w.F, s_ref, update_coords=True)
    C_ref = g.computeMaterialStiffness()
    with RVEServer(w.networks, w.strategies, precision=precision) as sv:
        for r in range(w.n_rve):
            sv.submit(r, w.F[r], update_coords=True, stiffness=True)
        res = sv.drain()
        sv.submit(0, np.eye(3), update_coords=False)
        plain = sv.drain()
    assert len(res) == w.n_rve
    for rec in res:
        r = int(rec["rve"])
        assert rec["status"] == 0 and rec["stiffness_status"] == 0
        np.testing.assert_array_equal(rec["sigma"], s_ref[r])
        np.testing.assert_array_equal(rec["C"], C_ref[r])
    assert plain["stiffness_status"][0] == -1 and not plain["C"][0].any()


def test_paged_server_evicts_and_matches_all_resident(lib_path):
    """Admission per request under a device-memory budget that holds two
    pages of two RVEs out of four pages: every round of updating requests
    evicts idle pages to host memory and re-admits saved ones, and every
    stress is bit-identical to one server holding all eight RVEs."""
    from mumfim_gb300 import synthetic as S
    from mumfim_gb300.serving import PagedRVEServer, RVEServer
    w = S.config2(n_rve=8, steps=400, n_min=400, n_max=3000)
    rounds = [[np.eye(3) + (S.uniform(S.param_seed(30 + k, r), 9) * 0.02 - 0.01).reshape(3, 3)
               for r in range(w.n_rve)] for k in range(3)]

    def run(sv):
        out = []
        for Fk in rounds:
            for r in range(w.n_rve):
                sv.submit(r, Fk[r], update_coords=True)
            res = sv.drain()
            assert len(res) == w.n_rve and (res["status"] == 0).all()
            s = np.zeros((w.n_rve, 6))
            s[res["rve"]] = res["sigma"]
            out.append(s)
        return out

    with RVEServer(w.networks, w.strategies, precision="mixed") as sv:
        ref = run(sv)
    from mumfim_gb300.serving import device_bytes_estimate
    pages = [w.networks[i:i + 2] for i in range(0, 8, 2)]
    budget = sum(sorted(device_bytes_estimate(p) for p in pages)[-2:]) * 1.001
    with PagedRVEServer(w.networks, w.strategies, hbm_budget_bytes=budget, page_size=2) as pv:
        got = run(pv)
        assert pv.evictions >= 6 and pv.admissions >= 8
        assert len(pv.resident) <= 2
    for a, b in zip(ref, got):
        np.testing.assert_array_equal(a, b)
