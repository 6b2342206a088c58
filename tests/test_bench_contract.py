"""The benchmark's command-line contract, checked on the CPU.

`bench.py --impl reference` times the reference's CPU path (the oracle port)
and prints one JSON line with the keys every arm prints; the GPU arm must
fail loudly, not fall back, when there is no GPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(args, timeout=300):
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                          capture_output=True, text=True, timeout=timeout)


def test_reference_arm_prints_one_contract_line():
    r = _run(["--impl", "reference", "--steps", "1", "--warmup", "3", "--n-rve", "8",
              "--cpu-sample-rves", "2", "--solve-steps", "100"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "fiber-steps/s" and d["unit"] == "fiber-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 3
    assert d["scaling"] == "weak" and d["vs_baseline"] is None
    assert d["ms_per_step"] > 0 and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["unit"] == d["unit"] and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_gpu_arm_fails_without_a_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = _run(["--n-rve", "4", "--solve-steps", "10", "--steps", "1", "--warmup", "3",
              "--no-extras", "--no-cpu-baseline"], timeout=120)
    assert r.returncode != 0
    assert not [x for x in r.stdout.splitlines() if x.startswith("{")]


def test_reference_arm_under_torchrun_prints_once():
    """With N ranks, rank 0 alone runs the reference arm and prints; the
    others exit 0 without work."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                        "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
                        str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "3", "--n-rve", "8",
                        "--cpu-sample-rves", "2", "--solve-steps", "100"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


def test_reference_arm_maps_no_product_library():
    """The reference arm generates its workload with the oracle's own build of
    the network generator and times the oracle: no library of the product is
    loaded into that process."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', "
            "'--warmup', '3', '--n-rve', '4', '--cpu-sample-rves', '1', '--solve-steps', '50']; "
            "runpy.run_path('bench.py', run_name='__main__'); "
            "print('MAPS', sorted({l.split()[-1] for l in open('/proc/self/maps') "
            "if l.rstrip().endswith('.so')}))")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    maps = [x for x in r.stdout.splitlines() if x.startswith("MAPS")][0]
    assert "oracle/_build/liboracle_fast.so" in maps
    assert "oracle/_build/libnetgen.so" in maps
    assert "mumfim_gb300/_lib" not in maps, maps


def test_autotune_candidates_and_sample():
    """The tuner's host logic: distinct candidate shapes, a sample that keeps
    the size mix, and a cache key that depends on the size mix."""
    from types import SimpleNamespace

    from mumfim_gb300.autotune import candidate_shapes, stratified_sample, workload_key
    shapes = candidate_shapes()
    assert len(shapes) == len(set(shapes)) == 12
    assert {s.small_rve_solve for s in shapes} == {"auto", "fiber"}
    assert {s.small_rve_solve for s in candidate_shapes(1.0)} == {"auto", "node"}
    assert len(set(candidate_shapes(0.5))) == 18
    nets = [SimpleNamespace(n_nodes=n, n_fibers=3 * n,
                            reactions=[SimpleNamespace(law=n % 2)]) for n in range(500, 5500, 5)]
    ids = stratified_sample(nets, 100)
    assert len(ids) == 100 and len(set(ids)) == 100
    sizes = sorted(nets[i].n_nodes for i in ids)
    assert sizes[0] < 600 and sizes[-1] > 5300
    assert workload_key(nets) == workload_key(list(reversed(nets)))
    assert workload_key(nets) != workload_key(nets[:300])
