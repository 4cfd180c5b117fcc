import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "component-based-2d-3d-nns-to-gpu-parallel-2d-3d-emst_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def fixtures():
    import numpy as np
    return np.load(os.path.join(GOLDEN, "reference_fixtures.npz"))


@pytest.fixture(scope="session")
def traces():
    import json
    with open(os.path.join(GOLDEN, "reference_traces.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree; a GPU test fails loudly if it is missing."""
    import emst_gb300
    if not os.path.exists(emst_gb300.LIB_PATH):
        emst_gb300.build()
    emst_gb300.lib()
    return emst_gb300
