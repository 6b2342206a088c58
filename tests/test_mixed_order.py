"""Host-side order of the mixed-precision RVEs (cluster_order, sell_layout in
mumfim_gb300/csrc/mfg_mixed_order.cpp), checked on the CPU: a small C++
program built from that file decodes every fiber end and every node-centric
incidence back to the network it came from, for clusters of 1, 2, 4 and 8
CTAs, and checks every index against its array."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "mumfim_gb300", "csrc")


def test_order_and_incidence_blocks_decode(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    from mumfim_gb300.build import _cuda_home
    try:
        cuda = _cuda_home()
    except RuntimeError:
        pytest.skip("CUDA headers not found")
    exe = str(tmp_path / "mixed_order_check")
    subprocess.run([gxx, "-O1", "-std=c++17", "-I" + CSRC, "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(cuda, "include"),
                    os.path.join(HERE, "native", "mixed_order_check.cpp"),
                    os.path.join(CSRC, "mfg_mixed_order.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad=0" in r.stdout
