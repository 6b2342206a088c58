"""The C-ABI library without a GPU: it loads, exports every declared entry
point, and rejects bad input on the host before touching a device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import REPO


def _declared_functions(header):
    src = open(os.path.join(REPO, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b(mfg_\w+)\s*\(", src,
                                 flags=re.M)))


def test_library_exports_every_declared_symbol(lib_path):
    """mumfim_gpu.h is the solver library's ABI, mumfim_netgen.h the network
    generator's; every header in include/ belongs to one of them."""
    from mumfim_gb300.build import NETGEN_PATH
    owner = {"mumfim_gpu.h": lib_path, "mumfim_netgen.h": NETGEN_PATH}
    headers = sorted(h for h in os.listdir(os.path.join(REPO, "include")) if h.endswith(".h"))
    assert headers == sorted(owner)
    for h, path in owner.items():
        lib = C.CDLL(path)
        names = _declared_functions(h)
        assert len(names) >= (25 if h == "mumfim_gpu.h" else 4)
        missing = [n for n in names if not hasattr(lib, n)]
        assert not missing, (h, missing)
    gpu = C.CDLL(lib_path)
    assert not hasattr(gpu, "mfg_generate_knn_network")


def test_status_strings_and_defaults(lib_path):
    import mumfim_gb300 as m
    from mumfim_gb300 import _abi
    L = m.load_library()
    assert L.mfg_abi_version() == 1
    assert L.mfg_status_string(3) == b"MFG_E_NOT_CONVERGED"
    s = _abi.mfg_strategy()
    L.mfg_default_strategy(C.byref(s))
    assert (s.visc_damp_coeff, s.crit_time_scale_factor, s.residual_tol, s.max_steps,
            s.mode) == (0.5, 0.8, 1e-6, 0, 0)


def _net(**kw):
    from mumfim_gb300 import FiberNetwork, Reaction
    c = np.array([[-0.5, 0, 0], [0.0, 0.1, 0], [0.5, 0, 0], [0.1, -0.2, 0.3]])
    conn = np.array([[0, 1], [1, 2], [1, 3], [3, 2]], dtype=np.int32)
    d = dict(coords=c, connectivity=conn, reactions=[Reaction(0, 1e-3, 1.0, 1.0)])
    d.update(kw)
    return FiberNetwork(d["coords"], d["connectivity"], d["reactions"])


@pytest.mark.parametrize("case,msg", [
    ("selfloop", "self-loop"), ("range", "outside"), ("zero", "zero length"),
    ("isolated", "no fibers"), ("modulus", "finite and > 0"), ("ramp0", "RAMP"),
    ("nan", "non-finite"), ("mismatch", "solution strategy"),
])
def test_invalid_input_is_rejected_on_the_host(lib_path, case, msg):
    import mumfim_gb300 as m
    from mumfim_gb300 import Reaction, SolutionStrategy
    net, strat = _net(), [SolutionStrategy()]
    if case == "selfloop":
        net = _net(connectivity=np.array([[0, 1], [1, 1]], dtype=np.int32))
    elif case == "range":
        net = _net(connectivity=np.array([[0, 1], [1, 9]], dtype=np.int32))
    elif case == "zero":
        c = np.array([[-0.5, 0, 0], [-0.5, 0, 0], [0.5, 0, 0]])
        net = _net(coords=c, connectivity=np.array([[0, 1], [1, 2]], dtype=np.int32))
    elif case == "isolated":
        c = np.array([[-0.5, 0, 0], [0.5, 0, 0], [0.1, 0.1, 0.1]])
        net = _net(coords=c, connectivity=np.array([[0, 1]], dtype=np.int32))
    elif case == "modulus":
        net = _net(reactions=[Reaction(0, 1e-3, -1.0, 1.0)])
    elif case == "ramp0":
        strat = [SolutionStrategy.ramp(0)]
    elif case == "nan":
        c = np.array([[-0.5, 0, 0], [np.nan, 0.1, 0], [0.5, 0, 0], [0.1, -0.2, 0.3]])
        net = _net(coords=c)
    elif case == "mismatch":
        strat = []
    with pytest.raises((m.MumfimGpuError, ValueError)) as ei:
        m.BatchedFiberRVEAnalysisExplicit([net], strat)
    assert msg in str(ei.value)
    if isinstance(ei.value, m.MumfimGpuError):
        assert ei.value.status == 1


def test_valid_input_without_gpu_reports_no_device(lib_path):
    import mumfim_gb300 as m
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(m.MumfimGpuError) as ei:
        m.BatchedFiberRVEAnalysisExplicit([_net()], [m.SolutionStrategy()])
    assert ei.value.status == 7


@pytest.mark.parametrize("field,value,msg", [
    ("max_cluster_ctas", 3, "max_cluster_ctas"), ("cluster_layout", 7, "cluster_layout"),
    ("precision", 5, "precision"), ("stiffness", 3, "stiffness"),
    ("small_rves_per_cta", 3, "small_rves_per_cta"), ("small_rve_solve", 3, "small_rve_solve"),
])
def test_bad_options_are_rejected_before_the_device(lib_path, field, value, msg):
    """Option checks come before any device call, so they hold on a machine
    without a GPU too."""
    from mumfim_gb300 import SolutionStrategy, _abi
    from mumfim_gb300.batched import load_library
    L = load_library()
    arr = _abi.NetworkArray([_net()], [SolutionStrategy()])
    o = _abi.mfg_options()
    L.mfg_default_options(C.byref(o))
    o.precision = 1
    setattr(o, field, value)
    h = C.c_void_p()
    assert L.mfg_batch_create(arr.nets, arr.strats, 1, C.byref(o), C.byref(h)) == 1
    assert msg in L.mfg_last_error().decode()
    assert not h.value
