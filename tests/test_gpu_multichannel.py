"""Multichannel data (X_t in R^n): residuals on the tensor cores and on the CUDA cores, the
theta update and the TSSolver against the FP64 oracle, which runs on the same BF16-rounded data
(the device stores X in BF16; parity is defined on those values).

Tolerances: b within 2e-6 of its scale (FP32 epilogue over a three-part BF16 theta, FP32
accumulation); theta within 5e-6 of its scale (FP32 products, 64-timestep FP32 partial sums
folded into FP64); at the TSSolver fixed point L within 1e-6 relative, theta within 1e-5 of its
scale and labels equal on >= 99.99% of timesteps."""
import numpy as np
import pytest

from pasc_inference_gb300 import PASC_PREC_MIXED, Problem, capi, datagen

pytestmark = pytest.mark.gpu


def _scale_rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


RES_CASES = [(1, 64, 2), (127, 64, 3), (128, 128, 8), (129, 128, 5), (5000, 128, 8), (3001, 256, 4),
             (1000, 64, 1), (777, 48, 3), (600, 200, 6)]


@pytest.mark.parametrize("T,n,K", RES_CASES)
def test_residual_engines_match_fp64(gpulib, oracle, T, n, K):
    rng = np.random.default_rng(T + n + K)
    X = datagen.bf16_round(rng.normal(size=T * n) + 0.5)
    theta = rng.normal(size=K * n)
    b_o = oracle.residual_b(X, theta, T, K, xdim=n)
    engines = [0, 1] if n in (64, 128, 256) else [1]
    with Problem(T, K, 10.0, precision=PASC_PREC_MIXED, xdim=n) as p:
        assert p.get_residual_engine() == engines[0]
        p.set_data(X)
        p.set_theta(theta)
        for e in engines:
            p.set_residual_engine(e)
            b = p.get_b()
            assert _scale_rel(b, b_o) <= 2e-6, (e, _scale_rel(b, b_o))
            p.update_b()
            assert np.array_equal(p.get_b(), b)  # deterministic


@pytest.mark.parametrize("T,n,K", [(5000, 128, 8), (1234, 64, 3), (3000, 256, 5), (999, 100, 2)])
def test_theta_update_matches_fp64(gpulib, oracle, T, n, K):
    rng = np.random.default_rng(T * K)
    X = datagen.bf16_round(rng.normal(size=T * n))
    g = rng.random(T * K)
    g = (g.reshape(T, K) / g.reshape(T, K).sum(axis=1, keepdims=True)).ravel()
    th_o = oracle.theta_update(g.astype(np.float32).astype(np.float64), X, T, K, xdim=n)
    with Problem(T, K, 10.0, precision=PASC_PREC_MIXED, xdim=n) as p:
        p.set_data(X)
        p.set_gamma(g)
        p.update_theta()
        th = p.get_theta()
    assert _scale_rel(th, th_o) <= 5e-6, _scale_rel(th, th_o)


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("T,n,K,eps2,stay", [(4000, 64, 4, 50.0, 0.99), (3000, 128, 8, 50.0, 0.995),
                                             (2500, 48, 3, 20.0, 0.99)])
def test_tssolver_tight_vs_oracle(gpulib, oracle, T, n, K, eps2, stay, variant):
    """From a uniform random gamma0 the first theta step makes the K centroids nearly equal,
    and (as in K-means) which fixed point the alternating loop then reaches depends on
    rounding; parity is checked from an informative start (true labels weighted 1 plus
    uniform [0, 1) noise on every cluster), where the fixed point is well defined."""
    mc = datagen.multichannel(T=T, n=n, K=K, seed=T + K, stay=stay, epssqr=eps2)
    g0 = mc.gamma0.reshape(K, T).copy()
    g0[mc.labels, np.arange(T)] += 1.0
    mc.gamma0 = g0.ravel()
    g_o, th_o, r_o, _ = oracle.tssolver_solve(mc.data, mc.gamma0, np.zeros(K * n), T, K, eps2, xdim=n,
                                              ts=oracle.ts_opts(maxit=300, eps=1e-13),
                                              spg=oracle.spg_opts(m=10, eps=1e-13, maxit=20000))
    with Problem(T, K, eps2, precision=PASC_PREC_MIXED, xdim=n) as p:
        p.set_sweep_variant(variant)  # both sweep kernels read the materialised b
        p.set_data(mc.data)
        p.set_gamma(mc.gamma0)
        p.set_theta(np.zeros(K * n))
        st = p.ts_solve(capi.ts_opts(maxit=300, eps=1e-13), capi.spgqp_opts(m=10, eps=1e-13, maxit=20000))
        th = p.get_theta()
        g = p.get_gamma()
    assert abs(st.L - r_o.L) <= 1e-6 * abs(r_o.L), (st.L, r_o.L)
    assert _scale_rel(th, th_o) <= 1e-5, _scale_rel(th, th_o)
    lab, lab_o = np.argmax(g.reshape(T, K), axis=1), np.argmax(g_o.reshape(T, K), axis=1)
    assert np.mean(lab == lab_o) >= 0.9999


def test_multichannel_consistency_200k(gpulib, oracle):
    """T = 2e5, n = 128, K = 8 with the reference's default stopping: gamma feasible, and the
    reported L equal to the objective of the returned gamma under the returned theta,
    evaluated in FP64 on the host from the BF16 data."""
    mc = datagen.multichannel(T=200_000, n=128, K=8, seed=4)
    T, n, K = mc.T, mc.n, mc.K
    with Problem(T, K, mc.epssqr, precision=PASC_PREC_MIXED, xdim=n) as p:
        p.set_data(mc.data)
        p.set_gamma(mc.gamma0)
        p.set_theta(np.zeros(K * n))
        st = p.ts_solve(capi.ts_opts(), capi.spgqp_opts(m=10))
        g = p.get_gamma()
        th = p.get_theta()
    G = g.reshape(T, K)
    assert np.all(G >= 0) and np.max(np.abs(G.sum(axis=1) - 1)) <= 1e-5
    b = oracle.residual_b(mc.data, th, T, K, xdim=n)
    L = 0.5 * g @ oracle.matmult(g, T, K, oracle.A_coeff(mc.epssqr, T)) - b @ g
    assert abs(L - st.L) <= 1e-6 * abs(L), (L, st.L)


def test_multichannel_argument_errors(gpulib):
    with pytest.raises(capi.PascError):
        Problem(100, 9, 1.0, precision=PASC_PREC_MIXED, xdim=64)  # K > 8
    with Problem(100, 3, 1.0, precision=PASC_PREC_MIXED, xdim=48) as p:
        with pytest.raises(capi.PascError):
            p.set_residual_engine(0)  # tensor cores need xdim in {64, 128, 256}
        with pytest.raises(capi.PascError):
            p.abserr_reconstructed(np.zeros(100))
    with Problem(100, 3, 1.0, precision=PASC_PREC_MIXED) as p:
        with pytest.raises(capi.PascError):
            p.set_residual_engine(1)  # 1-D data
