import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the CUDA library")


@pytest.fixture(scope="session")
def lib_path():
    from mumfim_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def golden_2_7():
    with open(os.path.join(GOLDEN, "network_2_7.json")) as fh:
        return json.load(fh)


def network_2_7(g):
    from mumfim_gb300.network_io import FiberNetwork, Reaction
    r = g["reaction"]
    return FiberNetwork(np.array(g["coords"], dtype=np.float64),
                        np.array(g["connectivity"], dtype=np.int32),
                        [Reaction(r["law"], r["radius"], r["youngs_modulus"], r["density"],
                                  r["B"], r["length_ratio_trns"])])


def voigt_to_mat(v):
    return np.array([[v[0], v[5], v[4]], [v[5], v[1], v[3]], [v[4], v[3], v[2]]])
