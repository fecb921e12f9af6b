"""Known-answer tests of the oracle that rest on mathematics, not on the reference's code:

1. projection onto the K-simplex (simplex_local.h:153-249): feasible blocks are returned
   unchanged, equal entries go to 1/K, a dominant entry to its vertex; random blocks agree with
   an independent sort-based projection (Held, Wolfe and Crowder 1974; Duchi et al. 2008) and
   satisfy the projection's optimality conditions;
2. the FEM-H1 operator (blockgraphsparse.cpp:51-109) for T = 1 .. 4 against the hand-assembled
   dense matrix (diagonal 2 at the ends and 4 inside, -2 next to it; 0 for T = 1);
3. SPG-QP on tiny problems against the optimality conditions of the QP over a product of
   simplices and against a general-purpose solver (SLSQP);
4. TSSolver on the golden fixtures (the reference's small_data test vector, the first 2000
   samples of its samplesignal, a synthetic T = 1e4 signal with levels {1, 2}): L never increases along the outer
   loop, and where the signal has levels {1, 2} theta ends near them."""
import numpy as np
import pytest


def _proj_sort(y):
    """Euclidean projection of one vector onto {z >= 0, sum z = 1} by sorting."""
    u = np.sort(y)[::-1]
    css = np.cumsum(u)
    j = np.arange(1, len(y) + 1)
    rho = np.nonzero(u - (css - 1.0) / j > 0)[0][-1]
    tau = (css[rho] - 1.0) / (rho + 1)
    return np.maximum(y - tau, 0.0)


def _projection_kkt_ok(x, y, tol):
    """y = max(x - tau, 0) for one tau, y feasible."""
    if np.any(y < 0) or abs(y.sum() - 1.0) > tol:
        return False
    on = y > 0
    tau = np.mean(x[on] - y[on])
    return bool(np.all(np.abs(x[on] - y[on] - tau) <= tol) and np.all(x[~on] <= tau + tol))


@pytest.mark.parametrize("K", [1, 2, 3, 4, 8])
def test_projection_keeps_feasible_blocks(oracle, K):
    # dyadic entries: the sum is exactly 1 in FP64, the reference's test for "already inside"
    rng = np.random.default_rng(K)
    blocks = []
    for _ in range(50):
        cuts = np.sort(rng.integers(0, 65, size=K - 1)) if K > 1 else np.array([], dtype=int)
        edges = np.concatenate(([0], cuts, [64]))
        blocks.append(np.diff(edges) / 64.0)
    x = np.concatenate(blocks)
    y = oracle.project(x, len(blocks), K)
    assert np.array_equal(y, x)


@pytest.mark.parametrize("K", [1, 2, 3, 5, 8, 13, 32])
def test_projection_equal_entries_and_vertices(oracle, K):
    cs = [-3.5, 0.0, 0.3, 7.0]
    x = np.concatenate([np.full(K, c) for c in cs])
    y = oracle.project(x, len(cs), K).reshape(len(cs), K)
    assert np.max(np.abs(y - 1.0 / K)) <= 1e-14
    # a dominant entry (at least 1 above every other) projects onto its vertex
    rng = np.random.default_rng(100 + K)
    T = 40
    x = rng.normal(size=(T, K)) * 2.0
    j = rng.integers(0, K, size=T)
    x[np.arange(T), j] = x.max(axis=1) + 1.0 + rng.random(T)
    y = oracle.project(x.ravel(), T, K).reshape(T, K)
    e = np.zeros((T, K))
    e[np.arange(T), j] = 1.0
    assert np.max(np.abs(y - e)) <= 1e-15


@pytest.mark.parametrize("K", [1, 2, 3, 5, 8, 13, 32])
def test_projection_random_blocks(oracle, K):
    rng = np.random.default_rng(7 * K)
    T = 200
    x = rng.normal(size=T * K) * 3.0
    x[: 10 * K] = rng.random(10 * K)  # some blocks near the simplex
    y = oracle.project(x, T, K).reshape(T, K)
    for t in range(T):
        xt = x[t * K:(t + 1) * K]
        assert np.max(np.abs(y[t] - _proj_sort(xt))) <= 1e-14, t
        assert _projection_kkt_ok(xt, y[t], 1e-13), t


def _dense_ahat(T):
    A = np.zeros((T, T))
    if T == 1:
        return A
    for t in range(T):
        if t > 0:
            A[t, t - 1] = -2.0
            A[t, t] += 2.0
        if t < T - 1:
            A[t, t + 1] = -2.0
            A[t, t] += 2.0
    return A


@pytest.mark.parametrize("T", [1, 2, 3, 4])
@pytest.mark.parametrize("K", [1, 2, 3])
def test_operator_against_dense_matrix(oracle, T, K):
    rng = np.random.default_rng(10 * T + K)
    x = rng.integers(-5, 6, size=T * K).astype(float)  # small integers: every sum is exact
    coeff = 0.5
    want = coeff * (_dense_ahat(T) @ x.reshape(T, K)).ravel()
    assert np.array_equal(oracle.matmult(x, T, K, coeff), want)
    if T >= 2:
        A = _dense_ahat(T)
        assert np.array_equal(np.diag(A), np.array([2.0] + [4.0] * (T - 2) + [2.0]))
        assert np.allclose(A.sum(axis=1), 0.0)


def _qp_kkt_residual(x, g, T, K):
    """Largest violation of the optimality conditions of min f over a product of simplices:
    per timestep, g_k equal to mu on the support and >= mu elsewhere, mu = min_k g_k."""
    X, G = x.reshape(T, K), g.reshape(T, K)
    mu = G.min(axis=1, keepdims=True)
    return float(np.max(np.where(X > 1e-9, G - mu, 0.0)))


@pytest.mark.parametrize("T,K,eps2,seed", [(2, 2, 1.0, 0), (3, 2, 5.0, 1), (3, 3, 0.5, 2), (5, 3, 2.0, 3),
                                           (6, 2, 20.0, 4), (4, 4, 1.0, 5)])
def test_spgqp_tiny_problems(oracle, T, K, eps2, seed):
    opt = pytest.importorskip("scipy.optimize")
    rng = np.random.default_rng(seed)
    data = rng.normal(size=T) + rng.integers(0, K, size=T)
    theta = np.sort(rng.normal(size=K) + np.arange(K))
    b = oracle.residual_b(data, theta, T, K)
    coeff = oracle.A_coeff(eps2, T)
    x0 = rng.random(T * K)
    x, r, _ = oracle.spgqp_solve(b, x0, T, K, coeff, oracle.spg_opts(m=10, eps=1e-15, maxit=20000))
    A = coeff * np.kron(_dense_ahat(T), np.eye(K))
    f = lambda z: 0.5 * z @ A @ z - b @ z  # noqa: E731
    assert abs(r.fx - f(x)) <= 1e-13 * max(1.0, abs(r.fx))
    g = A @ x - b
    scale = np.max(np.abs(b)) + np.max(np.abs(A @ x))
    assert _qp_kkt_residual(x, g, T, K) <= 1e-7 * scale
    assert np.all(x >= 0.0) and np.max(np.abs(x.reshape(T, K).sum(axis=1) - 1.0)) <= 1e-14
    cons = [{"type": "eq", "fun": (lambda z, t=t: z[t * K:(t + 1) * K].sum() - 1.0)} for t in range(T)]
    s = opt.minimize(f, np.full(T * K, 1.0 / K), jac=lambda z: A @ z - b, bounds=[(0.0, 1.0)] * (T * K),
                     constraints=cons, method="SLSQP", options={"ftol": 1e-15, "maxiter": 1000})
    assert f(x) <= s.fun + 1e-10 * max(1.0, abs(s.fun))
    assert abs(f(x) - s.fun) <= 1e-8 * max(1.0, abs(s.fun))


@pytest.mark.parametrize("case,levels", [(0, (1.0, 2.0)), (2, None), (3, (1.0, 2.0))])
def test_tssolver_fixtures_monotone_L(oracle, golden, case, levels):
    T, K, eps2 = (int(v) if i < 2 else float(v) for i, v in enumerate(golden[f"ts_{case}_TKe"]))
    data = golden[f"ts_{case}_data"]
    g0 = golden[f"ts_{case}_gamma0"]
    _, th, r, trL = oracle.tssolver_solve(data, g0, np.zeros(K), T, K, eps2,
                                          ts=oracle.ts_opts(maxit=200, eps=1e-12),
                                          spg=oracle.spg_opts(m=10, eps=1e-13, maxit=20000))
    assert len(trL) >= 2 and r.L_increased == 0
    assert np.all(np.diff(trL) <= 1e-12 * np.abs(trL[1:])), trL
    if levels is not None:
        assert np.max(np.abs(np.sort(th) - np.array(levels))) <= 0.05, th
