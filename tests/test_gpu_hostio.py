"""Host buffers through the C ABI: FP32 data and gamma (set_data_f32, set_gamma_f32,
get_gamma_f32) and page-locked host memory from pasc_gb300_host_alloc.

The FP32 calls must leave the device in the state the FP64 calls leave it in when given the
same values (widened to FP64): the same solve then follows bit for bit (objective and gamma
equal, not close)."""
import numpy as np
import pytest

from pasc_inference_gb300 import PASC_PREC_FP64, PASC_PREC_MIXED, Problem, capi, datagen

pytestmark = pytest.mark.gpu


def _signal(T, K, seed):
    sig = datagen.signal1d(T, K, np.linspace(0.0, 2.0, K), 50, 400, 0.5, seed)
    return sig.data.astype(np.float32), sig.gamma0.astype(np.float32)


@pytest.mark.parametrize("prec", [PASC_PREC_MIXED, PASC_PREC_FP64])
@pytest.mark.parametrize("T,K", [(5000, 3), (777, 5), (1, 2)])
def test_f32_host_buffers_equal_f64_calls(gpulib, prec, T, K):
    d32, g32 = _signal(T, K, T + K)
    theta = np.linspace(0.0, 2.0, K)
    opts = capi.spgqp_opts(m=10, maxit=40, stop_difff=0)
    res = []
    for f32 in (False, True):
        with Problem(T, K, 20.0, precision=prec) as p:
            if f32:
                p.set_data_f32(d32)
                p.set_gamma_f32(g32)
            else:
                p.set_data(d32.astype(np.float64))
                p.set_gamma(g32.astype(np.float64))
            p.permute_gamma()
            p.set_theta(theta)
            p.update_b()
            st = p.spgqp_solve(opts)
            out32 = np.empty(T * K, dtype=np.float32)
            p.get_gamma_f32_into(out32)
            res.append((st.fx, p.get_gamma(), out32, p.get_b()))
    (f0, g0, o0, b0), (f1, g1, o1, b1) = res
    assert f0 == f1
    np.testing.assert_array_equal(g0, g1)
    np.testing.assert_array_equal(o0, o1)
    np.testing.assert_array_equal(b0, b1)
    np.testing.assert_array_equal(o1, g1.astype(np.float32))
    if prec == PASC_PREC_MIXED:  # FP32 is the device format: nothing was rounded on the way
        np.testing.assert_array_equal(o1.astype(np.float64), g1)


def test_f32_multichannel_data(gpulib):
    T, n, K = 3000, 128, 4
    mc = datagen.multichannel(T=T, n=n, K=K, seed=9)
    x32 = mc.data.astype(np.float32)  # BF16 values are exact in FP32
    theta = np.random.default_rng(1).normal(size=K * n)
    bs = []
    for f32 in (False, True):
        with Problem(T, K, 10.0, precision=PASC_PREC_MIXED, xdim=n) as p:
            if f32:
                p.set_data_f32(x32)
            else:
                p.set_data(mc.data)
            p.set_theta(theta)
            bs.append(p.get_b())
    np.testing.assert_array_equal(bs[0], bs[1])


def test_sizes_are_checked(gpulib):
    with Problem(100, 3, 1.0) as p:
        with pytest.raises(capi.PascError):
            p.set_gamma_f32(np.zeros(299, dtype=np.float32))
        with pytest.raises(capi.PascError):
            p.set_data_f32(np.zeros(101, dtype=np.float32))
        with pytest.raises(capi.PascError):
            p.set_gamma(np.zeros(301))  # FP64 calls refuse another size too
        with pytest.raises(ValueError):
            p.get_gamma_f32_into(np.zeros(300, dtype=np.float64))


def test_page_locked_host_buffers(gpulib):
    T, K = 200_003, 3
    d32, g32 = _signal(T, K, 4)
    hb_d, hb_g, hb_o = capi.host_empty(T), capi.host_empty(T * K), capi.host_empty(T * K, np.float32)
    hb_d.array[:] = d32
    hb_g.array[:] = g32
    with Problem(T, K, 20.0, precision=PASC_PREC_MIXED) as p:
        p.set_data(hb_d.array)
        p.set_gamma(hb_g.array)
        p.permute_gamma()
        p.set_theta(np.array([0.0, 1.0, 2.0]))
        p.update_b()
        st = p.spgqp_solve(capi.spgqp_opts(m=10, maxit=30, stop_difff=0))
        p.get_gamma_f32_into(hb_o.array)
        ref = p.get_gamma()
    assert st.it == 30
    np.testing.assert_array_equal(hb_o.array.astype(np.float64), ref)
    for hb in (hb_d, hb_g, hb_o):
        hb.close()
        hb.close()  # a second close is harmless
    assert gpulib.pasc_gb300_host_free(None) == capi.PASC_OK
