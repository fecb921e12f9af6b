"""The vector level of the backend interface (pasc_gb300_vec_*, permute_f64, residual_f64,
theta_update_f64) on FP64 device buffers, through the C ABI, against numpy and the oracle.

Elementwise operations are FP64 in the reference's order: equal to numpy's results bit for
bit.  Reductions (dot, theta) sum in a block tree: within 1e-13 relative of the oracle's
sequential sums."""
import ctypes as C

import numpy as np
import pytest

from pasc_inference_gb300 import capi

pytestmark = pytest.mark.gpu


class DevVec:
    def __init__(self, L, n):
        self.L, self.n = L, n
        self.p = C.c_void_p()
        capi.check(L.pasc_gb300_vec_alloc(C.byref(self.p), n, 0))

    def set(self, a):
        capi.check(self.L.pasc_gb300_vec_set(self.p, np.ascontiguousarray(a, dtype=np.float64), self.n))

    def get(self):
        out = np.empty(self.n)
        capi.check(self.L.pasc_gb300_vec_get(self.p, out, self.n))
        return out

    def free(self):
        capi.check(self.L.pasc_gb300_vec_free(self.p))


def test_vector_operations(gpulib):
    L = gpulib
    n = 1_000_003
    rng = np.random.default_rng(3)
    x, y = rng.normal(size=n), rng.normal(size=n)
    vx, vy, vw = DevVec(L, n), DevVec(L, n), DevVec(L, n)
    assert np.all(vw.get() == 0.0)  # allocated zeroed
    vx.set(x)
    vy.set(y)
    np.testing.assert_array_equal(vx.get(), x)
    capi.check(L.pasc_gb300_vec_copy(vw.p, vx.p, n, None))
    np.testing.assert_array_equal(vw.get(), x)
    capi.check(L.pasc_gb300_vec_axpy(vw.p, -0.75, vy.p, n, None))  # w = x - 0.75 y
    np.testing.assert_array_equal(vw.get(), x + (-0.75) * y)
    capi.check(L.pasc_gb300_vec_waxpy(vw.p, 2.5, vx.p, vy.p, n, None))  # w = 2.5 x + y
    np.testing.assert_array_equal(vw.get(), 2.5 * x + y)
    capi.check(L.pasc_gb300_vec_scale(vw.p, -3.0, n, None))
    np.testing.assert_array_equal(vw.get(), -3.0 * (2.5 * x + y))
    d = C.c_double()
    capi.check(L.pasc_gb300_vec_dot(vx.p, vy.p, n, C.byref(d), None))
    ref = float(np.dot(x, y))
    assert abs(d.value - ref) <= 1e-12 * np.dot(np.abs(x), np.abs(y)), (d.value, ref)
    for v in (vx, vy, vw):
        v.free()


def test_model_steps_and_permutation(gpulib, oracle):
    L = gpulib
    T, K = 200_003, 3
    rng = np.random.default_rng(5)
    data = rng.normal(size=T) * 0.5 + rng.integers(0, K, size=T)
    theta = np.array([0.1, 1.05, 1.9])
    g_blocked = rng.random(T * K)
    vd, vt, vb, vg, vp = DevVec(L, T), DevVec(L, K), DevVec(L, T * K), DevVec(L, T * K), DevVec(L, T * K)
    vd.set(data)
    vt.set(theta)
    vg.set(g_blocked)
    bscale = oracle.b_coeff(T)
    capi.check(L.pasc_gb300_residual_f64(vd.p, vt.p, vb.p, T, K, bscale, None))
    np.testing.assert_array_equal(vb.get(), oracle.residual_b(data, theta, T, K))
    capi.check(L.pasc_gb300_permute_f64(vg.p, vp.p, T, K, None))
    g = oracle.permute_blocked_to_interleaved(g_blocked, T, K)
    np.testing.assert_array_equal(vp.get(), g)
    capi.check(L.pasc_gb300_theta_update_f64(vp.p, vd.p, vt.p, T, K, None))
    np.testing.assert_allclose(vt.get(), oracle.theta_update(g, data, T, K), rtol=1e-13, atol=0)
    assert L.pasc_gb300_permute_f64(vg.p, vg.p, T, K, None) == capi.PASC_ERR_ARG  # in place is refused
    for v in (vd, vt, vb, vg, vp):
        v.free()
