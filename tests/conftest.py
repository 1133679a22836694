import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) device and the built CUDA library")


@pytest.fixture(scope="session")
def golden():
    return {name: dict(np.load(os.path.join(GOLDEN, name + ".npz"))) for name in ("sobol", "acklam", "bridge", "books")}


@pytest.fixture(scope="session")
def gpu():
    """The CUDA engine; on a GPU run a missing library or device is a failure, not a skip."""
    import thoth_gb300 as G
    assert G.LIB_PATH.exists(), "libthoth_gpu.so not built (run __graft_entry__.build())"
    assert G.available(), "no usable sm_103 device: " + G.device_info()
    return G
