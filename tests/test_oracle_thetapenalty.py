"""The oracle's usethetainpenalty model (GraphH1FEMModel with theta in the penalty) on the CPU.
The reference implements it only in its PETSc specialisations (blockgraphsparse.cpp:161-185,
graphh1fem.cpp:154-160 and 306-380), which cannot be built here, so the pins are a literal
Python transcription of those loops on one rank, the unweighted limit (every block scaled by
the same coefficient) equal to the plain solver bit for bit, and the KKT conditions of the
final gamma for the block-scaled QP."""
import numpy as np
import pytest

from pasc_inference_gb300 import datagen


def _Ahat_rowsum(x, T, K):
    # MatMult with the assembled H1 stencil of one cluster block: 2x_t - x_{t-1} - x_{t+1}
    # on the interior, x_0 - x_1 and x_{T-1} - x_{T-2} at the ends, times 2
    X = x.reshape(T, K)
    Y = np.zeros_like(X)
    for t in range(T):
        s = 0.0
        if t > 0:
            s += 2.0 * X[t] - 2.0 * X[t - 1]
        if t < T - 1:
            s += 2.0 * X[t] - 2.0 * X[t + 1]
        Y[t] = s
    return Y


def _matmult_coeffs_transcribed(x, T, K, alpha, coeffs):
    """blockgraphsparse.cpp:161-185: y = MatMult(A, x); block k scaled by alpha*c_k*c_k."""
    Y = _Ahat_rowsum(x, T, K)
    for k in range(K):
        coeff = alpha * coeffs[k] * coeffs[k]
        Y[:, k] = coeff * Y[:, k]
    return Y.reshape(-1)


def _theta_penalty_transcribed(gamma, data, T, K, alpha):
    """graphh1fem.cpp:306-380 with usethetainpenalty: theta := 1, Agamma = A gamma,
    theta_k = (c gamma_k'x) / (c sum gamma_k + gamma_k'Agamma_k / 2), c = 1."""
    ones = np.ones(K)
    Ag = _matmult_coeffs_transcribed(gamma, T, K, alpha, ones).reshape(T, K)
    G = gamma.reshape(T, K)
    theta = np.zeros(K)
    coeff = 1.0
    for k in range(K):
        gAg = float(np.dot(G[:, k], Ag[:, k]))
        gx = float(np.dot(data, G[:, k]))
        gs = float(np.sum(G[:, k]))
        den = coeff * gs + 0.5 * gAg
        theta[k] = (coeff * gx) / den if den != 0 else 0.0
    return theta


@pytest.mark.parametrize("T,K", [(1, 2), (2, 3), (17, 2), (300, 4)])
def test_matmult_kc_transcription(oracle, T, K):
    rng = np.random.default_rng(T * 7 + K)
    x = rng.random(T * K)
    th = rng.random(K) * 3 - 1
    alpha = 0.37
    kc = np.array([alpha * th[k] * th[k] for k in range(K)])
    y = oracle.fem_h1_matmult_kc(x, T, K, kc)
    assert np.allclose(y, _matmult_coeffs_transcribed(x, T, K, alpha, th), rtol=1e-13, atol=1e-13)
    # all blocks with the same coefficient: the unweighted operator, bit for bit
    assert np.array_equal(oracle.fem_h1_matmult_kc(x, T, K, np.full(K, alpha)), oracle.matmult(x, T, K, alpha))


@pytest.mark.parametrize("T,K", [(1, 2), (5, 2), (400, 3), (1000, 5)])
def test_theta_penalty_transcription(oracle, T, K):
    rng = np.random.default_rng(T + 11 * K)
    g = rng.random(T * K)
    g = oracle.project(g, T, K)
    data = rng.standard_normal(T)
    for alpha in (0.0, 1e-3, 2.5):
        th = oracle.theta_update_penalty(g, data, T, K, alpha)
        assert np.allclose(th, _theta_penalty_transcribed(g, data, T, K, alpha), rtol=1e-12, atol=1e-14)
    # alpha = 0: the k-means update
    assert np.allclose(oracle.theta_update_penalty(g, data, T, K, 0.0), oracle.theta_update(g, data, T, K),
                       rtol=1e-12, atol=1e-14)


def test_theta_penalty_empty_cluster(oracle):
    T, K = 50, 3
    g = np.zeros(T * K)
    g[0::K] = 1.0  # cluster 1 and 2 empty: denominators 0
    data = np.linspace(-1, 1, T)
    th = oracle.theta_update_penalty(g, data, T, K, 0.5)
    assert th[1] == 0.0 and th[2] == 0.0
    assert th[0] == pytest.approx(np.sum(data) / T)


def test_spgqp_kc_uniform_equals_plain(oracle):
    T, K = 500, 3
    rng = np.random.default_rng(5)
    b = -rng.random(T * K)
    x0 = oracle.project(rng.random(T * K), T, K)
    coeff = 0.02
    o = oracle.spg_opts(maxit=300, eps=1e-12)
    xa, ra, _ = oracle.spgqp_solve(b, x0, T, K, coeff, o)
    xb, rb = oracle.spgqp_solve_kc(b, x0, T, K, np.full(K, coeff), o)
    assert np.array_equal(xa, xb) and ra.it == rb.it and ra.fx == rb.fx


def _kkt_residual(x, b, T, K, kc):
    g = _matmult_coeffs_transcribed(x, T, K, 1.0, np.sqrt(kc)) - b
    G = g.reshape(T, K)
    X = x.reshape(T, K)
    # on the simplex: g_k - mu_t >= 0 with equality where x_tk > 0, mu_t = min over the support
    worst = 0.0
    for t in range(T):
        sup = X[t] > 1e-9
        mu = G[t][sup].min()
        worst = max(worst, float(np.max(np.abs(G[t][sup] - mu))), float(max(0.0, mu - G[t].min())))
    return worst


def test_spgqp_kc_kkt(oracle):
    T, K = 300, 3
    rng = np.random.default_rng(9)
    b = -rng.random(T * K) * 0.1
    x0 = oracle.project(rng.random(T * K), T, K)
    kc = np.array([0.5, 0.05, 2.0])
    x, r = oracle.spgqp_solve_kc(b, x0, T, K, kc, oracle.spg_opts(maxit=20000, eps=1e-15))
    assert np.allclose(x.reshape(T, K).sum(axis=1), 1.0) and x.min() >= 0
    assert _kkt_residual(x, b, T, K, kc) < 1e-6
    fx = 0.5 * x @ _matmult_coeffs_transcribed(x, T, K, 1.0, np.sqrt(kc)) - b @ x
    assert r.fx == pytest.approx(fx, rel=1e-10, abs=1e-14)


def test_tssolver_model_limits(oracle):
    T, K = 2000, 3
    sig = datagen.signal1d(T, K, [0.0, 1.0, 2.0], 100, 400, 0.5, 3)
    g0 = sig.gamma0
    th0 = np.zeros(K)
    ts = oracle.ts_opts(maxit=30, eps=1e-9, init_permute=1)
    sp = oracle.spg_opts(maxit=500, eps=1e-10)
    # without the penalty flag the model run is the plain FEM-less run
    ga, tha, ra = oracle.tssolver_solve_fem(sig.data, g0, th0, T, K, 10.0, 1.0, ts=ts, spg=sp)
    gb, thb, rb = oracle.tssolver_solve_model(sig.data, g0, th0, T, K, 10.0, ts=ts, spg=sp)
    assert np.array_equal(ga, gb) and np.array_equal(tha, thb) and ra.L == rb.L
    # FEM coarsening together with the penalty flag is refused
    with pytest.raises(ValueError):
        oracle.tssolver_solve_model(sig.data, g0, th0, T, K, 10.0, fem_reduce=0.5, usethetainpenalty=True)


@pytest.mark.parametrize("epssqr", [1.0, 50.0])
def test_tssolver_penalty_run(oracle, epssqr):
    T, K = 3000, 3
    sig = datagen.signal1d(T, K, [0.0, 1.0, 2.0], 200, 600, 0.5, 21)
    g0 = sig.gamma0
    ts = oracle.ts_opts(maxit=60, eps=1e-10, init_permute=1)
    sp = oracle.spg_opts(maxit=3000, eps=1e-13)
    g, th, r = oracle.tssolver_solve_model(sig.data, g0, np.zeros(K), T, K, epssqr, usethetainpenalty=True,
                                           ts=ts, spg=sp)
    assert r.it_last >= 1 and np.isfinite(r.L)
    assert np.allclose(g.reshape(T, K).sum(axis=1), 1.0, atol=1e-12) and g.min() >= 0
    # the final gamma solves the block-scaled QP of the final theta
    alpha = oracle.A_coeff(epssqr, T)
    kc = np.array([alpha * th[k] * th[k] for k in range(K)])
    res = oracle.residual_b(sig.data, th, T, K)
    assert _kkt_residual(g, res, T, K, kc) < 1e-5
    # and the clustering still separates the levels
    lab = oracle.argmax_labels(g, T, K)
    truth = sig.labels
    agree = max(np.mean(np.array([p[l] for l in lab]) == truth) for p in _perms(K))
    assert agree > 0.9


def _perms(K):
    import itertools
    return list(itertools.permutations(range(K)))
