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


def fista_optimum(oracle, b, x0, T, K, coeff, iters=20000):
    """Independent FP64 optimum of min 1/2 x'Ax - b'x over the simplex product: accelerated
    projected gradient (step 1/L with L = 8*coeff >= lambda_max(A)) with gradient-based
    restart, built on the oracle's projection and operator.  Used where the reference's own
    SPG iteration is not a reliable optimum (tiny T, where its BB steps can stall)."""
    L = 8.0 * coeff if coeff > 0 else 1.0
    x = oracle.project(x0, T, K)
    y = x.copy()
    tk = 1.0

    def f(v):
        return 0.5 * v @ oracle.matmult(v, T, K, coeff) - b @ v

    for _ in range(iters):
        g = oracle.matmult(y, T, K, coeff) - b
        xn = oracle.project(y - g / L, T, K)
        if g @ (xn - x) > 0:  # restart the momentum when it points uphill
            tk = 1.0
            y = x.copy()
            continue
        tn = 0.5 * (1.0 + np.sqrt(1.0 + 4.0 * tk * tk))
        y = xn + ((tk - 1.0) / tn) * (xn - x)
        x, tk = xn, tn
    return f(x), x


@pytest.fixture(scope="session")
def qp_optimum(oracle):
    return lambda b, x0, T, K, coeff, iters=20000: fista_optimum(oracle, b, x0, T, K, coeff, iters)
