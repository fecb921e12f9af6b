"""The oracle against the reference's own code compiled here (oracle/_ref), on fresh random
cases.  Skipped where oracle/build_ref.sh finds no reference tree to compile (e.g. on a
machine that has only this repository)."""
import numpy as np
import pytest

from oracle import pasc_oracle as O


@pytest.fixture(scope="module")
def ref():
    O.build()
    if O.build_ref() is None:
        pytest.skip("oracle/_ref not built")
    return O


@pytest.mark.parametrize("K", [1, 2, 3, 6, 9, 40])
def test_projection_random(ref, K):
    rng = np.random.default_rng(K)
    T = 400
    x = rng.normal(size=T * K) * rng.choice([0.01, 1.0, 100.0], size=T * K)
    np.testing.assert_array_equal(ref.project(x, T, K), ref.ref_project(x, T, K))


@pytest.mark.parametrize("T,K,eps2,m", [(700, 2, 3.0, 20), (900, 3, 300.0, 10), (50, 7, 30.0, 5)])
def test_spgqp_random(ref, T, K, eps2, m):
    rng = np.random.default_rng(T + K)
    data = rng.normal(size=T) * 0.7 + rng.integers(0, K, size=T)
    b = ref.residual_b(data, np.linspace(0, K - 1, K), T, K)
    x0 = rng.random(T * K)
    coeff = ref.A_coeff(eps2, T)
    xr, it, hm, fx = ref.ref_spgqp_solve(b, x0, T, K, coeff, spgqpsolver_m=m)
    xo, r, _ = ref.spgqp_solve(b, x0, T, K, coeff, ref.spg_opts(m=m))
    assert (r.it, r.hessmult, r.fx) == (it, hm, fx)
    np.testing.assert_array_equal(xo, xr)


@pytest.mark.parametrize("eps2", [0.5, 20.0, 2000.0])
def test_tssolver_random(ref, eps2):
    rng = np.random.default_rng(int(eps2 * 10))
    T, K = 1500, 3
    data = np.repeat(rng.integers(0, 3, size=15), 100) + rng.normal(size=T) * 0.4
    g0 = rng.random(T * K)
    gr, thr, res = ref.ref_tssolver_solve(data, g0, np.zeros(K), T, K, eps2)
    go, tho, r, _ = ref.tssolver_solve(data, g0, np.zeros(K), T, K, eps2)
    assert r.L == res["L"] and r.it_last == res["it_last"] and r.aic == res["aic"]
    np.testing.assert_array_equal(go, gr)
    np.testing.assert_array_equal(tho, thr)


def test_tssolver_given_theta(ref):
    rng = np.random.default_rng(5)
    T, K = 800, 2
    data = np.repeat(rng.integers(1, 3, size=8), 100) + rng.normal(size=T) * 0.3
    g0 = rng.random(T * K)
    th0 = np.array([1.0, 2.0])
    gr, thr, res = ref.ref_tssolver_solve(data, g0, th0, T, K, 10.0, theta_given=True)
    go, tho, r, _ = ref.tssolver_solve(data, g0, th0, T, K, 10.0, ts=ref.ts_opts(thetasolved=1))
    assert r.L == res["L"]
    np.testing.assert_array_equal(go, gr)
    np.testing.assert_array_equal(tho, th0)


@pytest.mark.parametrize("nthreads", [2, 3, 5])
def test_spgqp_threads_follow_the_port(ref, nthreads):
    """With its vector operations split over threads, the reference's template sums in the
    oracle's chunk order: the same iterates as the port on as many threads (the timed CPU
    baseline runs this way on all cores), and one thread differs only by rounding."""
    rng = np.random.default_rng(nthreads)
    T, K = 30_000, 3
    data = np.repeat(rng.integers(0, K, size=30), 1000) + rng.normal(size=T) * 0.5
    b = ref.residual_b(data, np.arange(K, dtype=np.float64), T, K)
    x0 = rng.random(T * K)
    coeff = ref.A_coeff(10.0, T)
    kw = dict(spgqpsolver_m=10, spgqpsolver_maxit=40, spgqpsolver_stop_difff=0)
    xr, it, hm, fx = ref.ref_spgqp_solve(b, x0, T, K, coeff, nthreads=nthreads, **kw)
    xo, r, _ = ref.spgqp_solve(b, x0, T, K, coeff, ref.spg_opts(m=10, maxit=40, stop_difff=0), nthreads=nthreads)
    assert (r.it, r.hessmult, r.fx) == (it, hm, fx)
    np.testing.assert_array_equal(xo, xr)
    _, _, _, f1 = ref.ref_spgqp_solve(b, x0, T, K, coeff, nthreads=1, **kw)
    assert abs(f1 - fx) <= 1e-12 * abs(fx)


@pytest.mark.parametrize("T,K,eps2,m", [(1, 3, 10.0, 10), (2, 1, 10.0, 10), (5, 2, 1.0, 1), (3, 4, 1e4, 2)])
def test_spgqp_edge_sizes(ref, T, K, eps2, m):
    """One timestep (A = 0), one cluster (every point already feasible), GLL memory 1, a stiff
    few-timestep case: the oracle follows the reference's template bit for bit."""
    rng = np.random.default_rng(100 * T + K)
    data = rng.normal(size=T) + 1.0
    b = ref.residual_b(data, np.linspace(0, 2, K), T, K)
    x0 = rng.random(T * K)
    coeff = ref.A_coeff(eps2, T)
    xr, it, hm, fx = ref.ref_spgqp_solve(b, x0, T, K, coeff, spgqpsolver_m=m, spgqpsolver_maxit=200)
    xo, r, _ = ref.spgqp_solve(b, x0, T, K, coeff, ref.spg_opts(m=m, maxit=200))
    assert (r.it, r.hessmult, r.fx) == (it, hm, fx)
    np.testing.assert_array_equal(xo, xr)
