import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden_ref.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pasc_oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def gpulib():
    """The GPU library, built in-tree if needed; fails (never skips) when it cannot load."""
    from pasc_inference_gb300 import build as B, capi
    if not os.path.exists(capi.LIB_PATH):
        B.build()
    L = capi.load()
    assert L.pasc_gb300_device_count() >= 1, "no CUDA device visible"
    return L
