"""Multi-rank path on CPU: two gloo ranks shard a batch of RVEs, solve their
shards (the CPU oracle stands in for each rank's GPU), and all-gather the
stresses; the result must equal one process solving the whole batch."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from mumfim_gb300 import sharding
        from mumfim_gb300 import synthetic as S
        from oracle import pyoracle
        w = S.config2(n_rve=6, steps=200, n_min=200, n_max=900)
        shards = sharding.shard_rves([n.n_fibers for n in w.networks], world)
        mine = shards[rank]
        sub = w.subset(mine)
        rc, sig, st = pyoracle.OracleBatch(sub.networks, sub.strategies).run(sub.F)
        full = sharding.gather_stress(mine, sig, w.n_rve)
        q.put((rank, mine, full))
    finally:
        dist.destroy_process_group()


def test_two_rank_sharded_solve_equals_single_process(lib_path, oracle):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from mumfim_gb300 import synthetic as S
    w = S.config2(n_rve=6, steps=200, n_min=200, n_max=900)
    rc, sig, st = oracle.OracleBatch(w.networks, w.strategies).run(w.F)
    shards = sorted(r[1] for r in res)
    assert sorted(sum(shards, [])) == list(range(6)) and all(shards)
    for rank, mine, full in res:
        np.testing.assert_array_equal(full, sig)


def _liveness_worker(rank, world, port, q):
    """Step 0 on every rank; rank 2 then dies between steps; the survivors
    learn of it from the store before step 1 and stop with RankFailure."""
    import time
    from datetime import timedelta

    import torch.distributed as dist
    from mumfim_gb300 import sharding
    store = dist.TCPStore("127.0.0.1", port, world, rank == 0, timedelta(seconds=60))
    sharding.await_peers(store, "step0", rank, world, timeout_s=30)
    if rank == 2:
        os._exit(3)  # a crashed rank: no cleanup, no goodbye
    t0 = time.monotonic()
    try:
        sharding.await_peers(store, "step1", rank, world, timeout_s=3)
        q.put((rank, None, time.monotonic() - t0))
    except sharding.RankFailure as e:
        q.put((rank, e.missing, time.monotonic() - t0))
    # rank 0 hosts the store's server: it stays up until rank 1's last store
    # operation has been acknowledged
    if rank == 1:
        store.set("bye/1", b"1")
    else:
        store.wait(["bye/1"], timedelta(seconds=30))


def test_dead_rank_is_detected_between_steps():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_liveness_worker, args=(r, 3, port, q)) for r in range(3)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
    assert procs[2].exitcode == 3
    assert procs[0].exitcode == 0 and procs[1].exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    for rank, missing, waited in res:
        assert missing == [2]
        assert waited < 30


def test_shard_balance():
    from mumfim_gb300.sharding import shard_rves
    work = [10, 9, 8, 7, 6, 5, 4, 3, 2, 1]
    s = shard_rves(work, 3)
    loads = [sum(work[i] for i in sh) for sh in s]
    assert sorted(sum(s, [])) == list(range(10))
    assert max(loads) - min(loads) <= 1
    with pytest.raises(ValueError):
        shard_rves(work, 0)
