import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def h2o():
    """H2O/STO-3G integrals and RHF for the three basis variants of the reference inputs."""
    import gaussian_ints as g

    cache = {}

    def get(basis):
        if basis not in cache:
            cache[basis] = g.h2o_sto3g(basis)
        return cache[basis]

    return get


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", "h2o_sto3g_golden.npz"))
