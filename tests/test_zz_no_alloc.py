"""The allocation-free theta update (pasc_gb300_theta_update_noalloc), for callers that cannot
allocate device memory when they need the theta step -- hosts whose device memory belongs to
another framework's allocator, real-time loops that allow no allocation after start-up.  It is checked through the C ABI against the
problem-handle path (pasc_gb300_update_theta), which computes the same reduction with scratch
the handle allocated: relative difference <= 1e-12 (both sum the same FP32 values in the same
order, so the results are expected to be identical).  Two calls in a row share the static
scratch; the second must not see the first's leftovers.  This file is collected last so that
a stop at its first failure has already run every other test; it also passes on its own in a
fresh process (its first call does the one-time set-up)."""
import ctypes as C

import numpy as np
import pytest

from pasc_inference_gb300 import PASC_PREC_MIXED, Problem, capi, datagen

pytestmark = pytest.mark.gpu


def _reference_theta(gamma32, data32, T, K):
    with Problem(T, K, 1.0, precision=PASC_PREC_MIXED) as p:
        p.set_data(data32.astype(np.float64))
        p.set_gamma(gamma32.astype(np.float64))
        p.update_theta()
        return p.get_theta()


def test_theta_update_noalloc_matches_update_theta(gpulib):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    for T, K, seed in [(1_000_003, 3, 1), (4099, 8, 2)]:  # two calls in a row
        sig = datagen.signal1d(T, K, np.linspace(0.0, 2.0, K), max(T // 200, 1), max(T // 20, 2), 0.5, seed)
        gamma32 = datagen.normalised_gamma(sig.gamma0, T, K).astype(np.float32)
        data32 = sig.data.astype(np.float32)
        ref = _reference_theta(gamma32, data32, T, K)
        g = torch.tensor(gamma32, device="cuda")
        d = torch.tensor(data32, device="cuda")
        out = torch.full((K,), float("nan"), dtype=torch.float64, device="cuda")
        rc = gpulib.pasc_gb300_theta_update_noalloc(C.c_void_p(g.data_ptr()), C.c_void_p(d.data_ptr()),
                                                    T, K, C.c_void_p(out.data_ptr()), None)
        assert rc == capi.PASC_OK, gpulib.pasc_gb300_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got))
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0.0)


def test_theta_update_noalloc_rejects_k_beyond_its_scratch(gpulib):
    torch = pytest.importorskip("torch")
    g = torch.zeros(90, dtype=torch.float32, device="cuda")
    d = torch.zeros(10, dtype=torch.float32, device="cuda")
    out = torch.zeros(9, dtype=torch.float64, device="cuda")
    rc = gpulib.pasc_gb300_theta_update_noalloc(C.c_void_p(g.data_ptr()), C.c_void_p(d.data_ptr()), 10, 9,
                                                C.c_void_p(out.data_ptr()), None)
    assert rc == capi.PASC_ERR_ARG
    assert b"[1, 8]" in gpulib.pasc_gb300_last_error()
