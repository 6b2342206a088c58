"""The integration shim of INTEGRATION.md, compiled and run.

The C++ class a mumfim maintainer adds (BatchedFiberRVEAnalysisGB300) is read
out of INTEGRATION.md as written, compiled against stand-ins for the mumfim,
Kokkos and APF declarations it uses (tests/native/mumfim_mock), and driven by
tests/native/shim_check.cpp through libmumfim_gpu.so.

The networks are the reference's Network_2_7 with its damping (100), once
with reaction 0 linear and once with reaction 0 a NonlinearReaction. The
reference's batched analysis runs the linear law on reaction 0's E, A and
rho whatever its type (BatchedFiberRVEAnalysisExplicit.h:202-212), and the
shim's default policy does the same; its NetworkLaw policy forwards B and
the transition ratio instead.
"""
import json
import math
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import REPO, network_2_7

NATIVE = os.path.join(REPO, "tests", "native")


def _shim_source() -> str:
    with open(os.path.join(REPO, "INTEGRATION.md")) as fh:
        text = fh.read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, flags=re.S)
    shim = [b for b in blocks if "class BatchedFiberRVEAnalysisGB300" in b]
    assert len(shim) == 1, "INTEGRATION.md must hold exactly one shim code block"
    return shim[0]


@pytest.fixture(scope="module")
def shim_exe(lib_path, tmp_path_factory):
    d = tmp_path_factory.mktemp("shim")
    (d / "BatchedFiberRVEAnalysisGB300.h").write_text(_shim_source())
    exe = d / "shim_check"
    lib_dir = os.path.dirname(lib_path)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-Wno-unused-function",
           "-I", str(d), "-I", os.path.join(NATIVE, "mumfim_mock"),
           "-I", os.path.join(REPO, "include"), os.path.join(NATIVE, "shim_check.cpp"),
           "-o", str(exe), "-L", lib_dir, "-lmumfim_gpu", f"-Wl,-rpath,{lib_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def _write_input(path, golden, variants):
    """variants: (law, B, lt, cmp) per RVE on Network_2_7."""
    rc = golden["reaction"]
    X = np.array(golden["coords"])
    conn = np.array(golden["connectivity"], dtype=np.int64)
    F = np.array(golden["F"])
    lines = [str(len(variants))]
    for law, B, lt, cmp in variants:
        lines.append(f"{law} {rc['youngs_modulus']!r} {rc['radius']!r} {rc['density']!r} "
                     f"{B!r} {lt!r} {cmp!r} 1.0 {golden['visc_damp_coeff']!r} "
                     f"{len(X)} {len(conn)}")
        lines += [" ".join(repr(float(v)) for v in p) for p in X]
        lines += [f"{a} {b}" for a, b in conn]
        lines.append(" ".join(repr(float(v)) for v in F))
    path.write_text("\n".join(lines) + "\n")


def _run(exe, mode, policy, inp):
    r = subprocess.run([exe, mode, policy, str(inp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout.strip()


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


NONLINEAR = (1, 5.0, 1.05, 1.0)
LINEAR = (0, 0.0, 0.0, 1.0)


def test_shim_compiles_and_validates_a_nonlinear_network(shim_exe, golden_2_7, tmp_path):
    """Both policies get through the library's argument checks for a network
    whose reaction 0 is nonlinear; on a machine without a GPU the create call
    then stops at the device check. An unsupported compressive transition
    ratio is refused by the shim."""
    inp = tmp_path / "in.txt"
    _write_input(inp, golden_2_7, [NONLINEAR, LINEAR])
    for policy in ("reference", "network"):
        out = _run(shim_exe, "create", policy, inp)
        if _has_gpu():
            assert out == "created", out
        else:
            assert out.startswith("mumfim_error: no CUDA device"), out
    _write_input(inp, golden_2_7, [(1, 5.0, 1.05, 0.9)])
    out = _run(shim_exe, "create", "network", inp)
    assert "compressive transition ratio of 1.0 only" in out
    out = _run(shim_exe, "create", "reference", inp)
    assert "compressive" not in out


@pytest.mark.gpu
@pytest.mark.parametrize("policy", ["reference", "network"])
def test_shim_solves_like_the_python_binding(shim_exe, golden_2_7, tmp_path, policy):
    """Stress, stiffness and orientation from the shim equal the Python
    binding's on the same networks, with the law the policy selects: linear
    for both RVEs under the reference policy, the nonlinear law for RVE 0
    under the network-law policy."""
    import mumfim_gb300 as m
    from mumfim_gb300.network_io import Reaction
    inp = tmp_path / "in.txt"
    _write_input(inp, golden_2_7, [NONLINEAR, LINEAR])
    res = json.loads(_run(shim_exe, "solve", policy, inp))
    g = golden_2_7
    rc = g["reaction"]
    radius = math.sqrt(rc["radius"] * rc["radius"] * math.pi / math.pi)  # what the shim passes
    nets = []
    for law, B, lt, _ in (NONLINEAR, LINEAR):
        net = network_2_7(g)
        use_nl = policy == "network" and law == 1
        net.reactions = [Reaction(1 if use_nl else 0, radius, rc["youngs_modulus"], rc["density"],
                                  B if use_nl else 0.0, lt if use_nl else 0.0)]
        nets.append(net)
    strat = [m.SolutionStrategy(visc_damp_coeff=g["visc_damp_coeff"], crit_time_scale_factor=0.8,
                                residual_tol=1e-6)] * 2
    py = m.BatchedFiberRVEAnalysisExplicit(nets, strat)
    F = np.repeat(np.array(g["F"]).reshape(1, 3, 3), 2, 0)
    sig = np.zeros((2, 6))
    py.run(F, sig)
    C = py.computeMaterialStiffness()
    om = py.compute3DOrientationTensor()
    np.testing.assert_array_equal(np.array(res["sigma"]).reshape(2, 6), sig)
    np.testing.assert_array_equal(np.array(res["C"]).reshape(2, 6, 6), C)
    np.testing.assert_array_equal(np.array(res["omega"]).reshape(2, 3, 3), om)
    if policy == "reference":
        np.testing.assert_array_equal(sig[0], sig[1])
    else:
        assert not np.array_equal(sig[0], sig[1])
