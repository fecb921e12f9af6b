"""The oracle's adjoint (derivatives of a loss through the converged gamma-step QP) pinned on
the CPU.  The reference has no adjoint, so the pins are mathematical: the adjoint vector
against a dense solve of the projected system, and the gradients against central finite
differences (step 1e-4 relative) of the loss through exact QP solutions.

Exact QP solutions: a first-order solve (the oracle's SPG, tight) finds the active set; the
equality-constrained QP on that free set is then solved with dense linear algebra (KKT
system), and the result is accepted only if it satisfies the full optimality conditions
(free entries positive, multipliers of the active bounds non-negative)."""
import numpy as np
import pytest

from pasc_inference_gb300 import datagen


def _dense_A(T, K, coeff):
    L = np.zeros((T, T))
    for t in range(T):
        if t > 0:
            L[t, t] += 2.0
            L[t, t - 1] -= 2.0
        if t < T - 1:
            L[t, t] += 2.0
            L[t, t + 1] -= 2.0
    return coeff * np.kron(L, np.eye(K))


def exact_qp(oracle, b, x0, T, K, coeff, act_tol=1e-9):
    """Solution of min 1/2 x'Ax - b'x over the simplex product, exact to rounding."""
    x, _, _ = oracle.spgqp_solve(b, x0, T, K, coeff, oracle.spg_opts(m=10, eps=1e-15, maxit=20000))
    A = _dense_A(T, K, coeff)
    for _ in range(5):
        free = x > act_tol
        fi = np.flatnonzero(free)
        C = np.zeros((T, len(fi)))
        for j, i in enumerate(fi):
            C[i // K, j] = 1.0
        keep = C.sum(axis=1) > 0
        C = C[keep]
        n, m = len(fi), C.shape[0]
        KKT = np.block([[A[np.ix_(fi, fi)], C.T], [C, np.zeros((m, m))]])
        rhs = np.concatenate([b[fi], np.ones(m)])
        sol = np.linalg.solve(KKT, rhs)
        xn = np.zeros(T * K)
        xn[fi] = sol[:n]
        # multipliers: A x - b + nu_t - mu = 0  ->  mu = A x - b + nu_t on the active entries
        nu = np.zeros(T)
        nu[np.flatnonzero(keep)] = sol[n:]
        mu = A @ xn - b + np.repeat(nu, K)
        ok_free = np.all(xn[fi] > 0.0)
        ok_mu = np.all(mu[~free] >= -1e-12 * max(1.0, np.abs(b).max()))
        if ok_free and ok_mu:
            return xn
        x = np.maximum(xn, 0.0) if not ok_free else xn
        if not ok_mu:
            x[(~free) & (mu < 0)] = 1e-3  # free the violated bound and re-solve
        x = oracle.project(x, T, K)
    raise AssertionError("active set did not settle")


def _case(T, K, eps2, seed, oracle):
    sig = datagen.signal1d(T, K, np.linspace(0.0, K - 1.0, K), max(T // 8, 2), max(T // 3, 3), 0.35, seed)
    theta = np.linspace(0.0, K - 1.0, K) + 0.05
    b = oracle.residual_b(sig.data, theta, T, K)
    coeff = oracle.A_coeff(eps2, T)
    x = exact_qp(oracle, b, oracle.project(sig.gamma0.copy(), T, K), T, K, coeff)
    return sig, theta, b, coeff, x


def _loss(oracle, data, theta, clean, T, K, eps2, x0):
    b = oracle.residual_b(data, theta, T, K)
    x = exact_qp(oracle, b, x0, T, K, oracle.A_coeff(eps2, T))
    return oracle.recon_mse(x, theta, clean, T, K)[0], x


@pytest.mark.parametrize("T,K,eps2,seed", [(40, 3, 20.0, 1), (60, 2, 50.0, 2), (30, 4, 5.0, 3)])
def test_adjoint_vector_matches_dense_solve(oracle, T, K, eps2, seed):
    sig, theta, b, coeff, x = _case(T, K, eps2, seed, oracle)
    _, dg, _ = oracle.recon_mse(x, theta, sig.clean, T, K)
    deps, dX, dth, lam, r = oracle.adjoint(x, sig.data, theta, dg, T, K, eps2, cg_tol=1e-14)
    assert r.status == 1
    # orthonormal basis of S: per timestep with free set F, an orthonormal basis of the
    # zero-sum vectors supported on F
    cols = []
    free = x > 1e-7
    for t in range(T):
        F = [k for k in range(K) if free[t * K + k]]
        for j in range(1, len(F)):
            v = np.zeros(T * K)
            for q in range(j):
                v[t * K + F[q]] = 1.0
            v[t * K + F[j]] = -float(j)
            cols.append(v / np.linalg.norm(v))
    assert len(cols) == r.free_dims
    if not cols:
        assert np.all(lam == 0.0)
        return
    B = np.array(cols).T
    A = _dense_A(T, K, coeff)
    lam_dense = B @ np.linalg.solve(B.T @ A @ B, B.T @ dg)
    assert np.max(np.abs(lam - lam_dense)) <= 1e-9 * np.max(np.abs(lam_dense))


@pytest.mark.parametrize("T,K,eps2,seed", [(40, 3, 20.0, 1), (60, 2, 50.0, 2), (30, 4, 5.0, 3)])
def test_adjoint_gradients_match_finite_differences(oracle, T, K, eps2, seed):
    sig, theta, b, coeff, x = _case(T, K, eps2, seed, oracle)
    loss0, dg, dth_direct = oracle.recon_mse(x, theta, sig.clean, T, K)
    deps, dX, dth, lam, r = oracle.adjoint(x, sig.data, theta, dg, T, K, eps2, cg_tol=1e-14)
    assert r.free_dims > 0, "case has no free directions: nothing is checked"

    h = 1e-4
    # epssqr
    lp, xp = _loss(oracle, sig.data, theta, sig.clean, T, K, eps2 * (1 + h), x)
    lm, xm = _loss(oracle, sig.data, theta, sig.clean, T, K, eps2 * (1 - h), x)
    assert np.array_equal(xp > 1e-7, x > 1e-7) and np.array_equal(xm > 1e-7, x > 1e-7)
    fd = (lp - lm) / (2 * h * eps2)
    assert abs(fd - deps) <= 1e-6 * abs(deps) + 1e-13, (fd, deps)
    # data, along a random direction
    v = np.random.default_rng(seed).normal(size=T)
    hx = h * np.max(np.abs(sig.data))
    lp, _ = _loss(oracle, sig.data + hx * v, theta, sig.clean, T, K, eps2, x)
    lm, _ = _loss(oracle, sig.data - hx * v, theta, sig.clean, T, K, eps2, x)
    fd = (lp - lm) / (2 * hx)
    assert abs(fd - dX @ v) <= 1e-6 * np.abs(dX).sum() * np.abs(v).max() + 1e-13, (fd, dX @ v)
    # theta (through b and the loss itself)
    for k in range(K):
        e = np.zeros(K)
        e[k] = h
        lp, _ = _loss(oracle, sig.data, theta + e, sig.clean, T, K, eps2, x)
        lm, _ = _loss(oracle, sig.data, theta - e, sig.clean, T, K, eps2, x)
        fd = (lp - lm) / (2 * h)
        an = dth[k] + dth_direct[k]
        assert abs(fd - an) <= 1e-6 * np.abs(dth + dth_direct).max() + 1e-13, (k, fd, an)


def test_adjoint_vertex_solution_has_zero_gradient(oracle):
    """A solution with every timestep at a vertex (noise-free data, long segments, weak
    regularisation): no free direction, so the QP solution is locally constant and every
    derivative through it is zero."""
    T, K, eps2 = 30, 3, 0.01
    labels = np.repeat([0, 1, 2], 10)
    theta = np.array([0.0, 1.0, 2.0])
    data = theta[labels]
    b = oracle.residual_b(data, theta, T, K)
    gamma = exact_qp(oracle, b, np.full(T * K, 1.0 / K), T, K, oracle.A_coeff(eps2, T))
    assert np.array_equal(gamma, np.eye(K)[labels].ravel())
    dg = np.random.default_rng(0).normal(size=T * K)
    deps, dX, dth, lam, r = oracle.adjoint(gamma, data, theta, dg, T, K, eps2)
    assert r.free_dims == 0 and r.status == 1
    assert deps == 0.0 and np.all(dX == 0.0) and np.all(dth == 0.0)


@pytest.mark.parametrize("T,K,eps2,seed", [(40, 3, 20.0, 1), (60, 2, 50.0, 2)])
def test_free_set_read_through_a_projected_step(oracle, T, K, eps2, seed):
    """An inexact end point whose active entries are small positives (as an FP32 iterate
    x^c + beta d leaves them) yields the free set of the exact solution, and nearly its
    gradient: the free set is taken from Proj(gamma - a g), not from gamma itself."""
    sig, theta, b, coeff, x = _case(T, K, eps2, seed, oracle)
    _, dg, _ = oracle.recon_mse(x, theta, sig.clean, T, K)
    deps, dX, _, _, r = oracle.adjoint(x, sig.data, theta, dg, T, K, eps2)
    xn = x.copy()
    xn[x == 0.0] = 1e-6
    xn = (xn.reshape(T, K) / xn.reshape(T, K).sum(axis=1, keepdims=True)).ravel()
    deps_n, dX_n, _, _, r_n = oracle.adjoint(xn, sig.data, theta, dg, T, K, eps2)
    assert r_n.free_dims == r.free_dims
    assert abs(deps_n - deps) <= 1e-3 * abs(deps)
