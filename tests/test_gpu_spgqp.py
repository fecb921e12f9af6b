"""SPG-QP solves on the GPU (both precisions) through the C ABI against the FP64 oracle and
the reference-produced golden vectors.

Tolerances (written per test): the fp64 path follows the reference's operation order but
sums its dot products in a different (tree) order, so trajectories agree to ~1e-13 relative
over the first iterations and converged objectives to 1e-9 relative.  The mixed path keeps
gamma and the gradient in FP32: converged objectives within 1e-6 relative of FP64 (the
accuracy target of the path), gamma within 2e-3 absolute where the FP64 problem is
well-conditioned."""
import numpy as np
import pytest

from pasc_inference_gb300 import PASC_PREC_FP64, PASC_PREC_MIXED, Problem, capi

pytestmark = pytest.mark.gpu


def _qp(T, K, eps2, seed, oracle):
    rng = np.random.default_rng(seed)
    data = rng.normal(size=T) * 0.5 + rng.integers(0, K, size=T)
    theta = np.arange(K, dtype=float)
    x0 = rng.random(T * K)
    b = oracle.residual_b(data, theta, T, K)
    return data, theta, x0, b, oracle.A_coeff(eps2, T)


def _problem(T, K, eps2, data, theta, x0, prec):
    p = Problem(T, K, eps2, precision=prec)
    p.set_data(data)
    p.set_theta(theta)
    p.set_gamma(x0)
    p.update_b()
    return p


@pytest.mark.parametrize("T,K", [(1000, 2), (777, 3), (300, 5), (64, 8)])
def test_fp64_first_iterations_match_oracle(gpulib, oracle, T, K):
    data, theta, x0, b, coeff = _qp(T, K, 30.0, T + K, oracle)
    for maxit in (0, 1, 2, 5):
        xo, ro, _ = oracle.spgqp_solve(b, x0, T, K, coeff, oracle.spg_opts(maxit=maxit))
        with _problem(T, K, 30.0, data, theta, x0, PASC_PREC_FP64) as p:
            st = p.spgqp_solve(capi.spgqp_opts(maxit=maxit))
            assert st.it == ro.it
            assert abs(st.fx - ro.fx) <= 1e-13 * abs(ro.fx)
            np.testing.assert_allclose(p.get_gamma(), xo, rtol=0, atol=1e-12)


def _golden_spg(golden):
    n = len({k.split("_")[1] for k in golden.files if k.startswith("spg_")})
    for i in range(n):
        T, K, coeff = golden[f"spg_{i}_TKc"]
        T, K = int(T), int(K)
        kw = {}
        for nm, v in zip(golden[f"spg_{i}_optnames"], golden[f"spg_{i}_optvals"]):
            nm = str(nm)
            if nm:
                f = nm.replace("spgqpsolver_", "")
                kw[f] = int(v) if f in ("m", "maxit", "stop_difff", "stop_normgp") else float(v)
        yield i, T, K, coeff * T, kw


@pytest.mark.parametrize("prec", [PASC_PREC_FP64, PASC_PREC_MIXED])
def test_golden_solves(gpulib, golden, oracle, qp_optimum, prec):
    """The reference-produced SPG solves.  The GPU forms the same b from the same data and
    theta.  Fixed-length runs (maxit < 100) must follow the reference's trajectory
    (1e-12 relative fp64, 2e-6 mixed).  Runs the reference stopped on |f - f_old| < eps sit
    somewhere short of the optimum, so there the check is that the GPU driven to the optimum
    matches the oracle's optimum (1e-9 fp64, 1e-6 mixed) and is no worse than the
    reference's stopped objective.  The optimum is an independent FP64 solve (accelerated
    projected gradient): on the 2-timestep case the reference's iteration, continued past
    convergence, leaves the optimum (its BB step blows up as d'Ad -> 0)."""
    for i, T, K, eps2, kw in _golden_spg(golden):
        if T == 1:
            # A = 0: the reference divides by d'Ad = 0 and ends at an infeasible point; the GPU
            # answer is checked against the analytic optimum in test_edge_sizes
            continue
        data, theta = golden[f"spg_{i}_data"], golden[f"spg_{i}_theta"]
        b = golden[f"spg_{i}_b"]
        np.testing.assert_array_equal(oracle.residual_b(data, theta, T, K), b)
        it_ref, _, fx_ref = golden[f"spg_{i}_res"]
        x0 = golden[f"spg_{i}_x0"]
        fixed = kw.get("maxit", 1000) < 100
        with _problem(T, K, eps2, data, theta, x0, prec) as p:
            if fixed:
                st = p.spgqp_solve(capi.spgqp_opts(**kw))
                assert st.it == int(it_ref)
                tol = 1e-12 if prec == PASC_PREC_FP64 else 2e-6
                assert abs(st.fx - fx_ref) <= tol * abs(fx_ref), (i, st.fx, fx_ref)
                continue
            tight = {k: v for k, v in kw.items() if k not in ("eps", "stop_normgp", "stop_difff", "maxit")}
            st = p.spgqp_solve(capi.spgqp_opts(maxit=4000, stop_difff=0, **tight))
        coeff = oracle.A_coeff(eps2, T)
        f_opt, _ = qp_optimum(b, x0, T, K, coeff)
        tol = 1e-9 if prec == PASC_PREC_FP64 else 1e-6
        assert abs(st.fx - f_opt) <= tol * abs(f_opt), (i, st.fx, f_opt)
        assert fx_ref >= f_opt - 1e-12 * abs(f_opt)  # the reference's stopped objective


@pytest.mark.parametrize("T,K,eps2", [(1000, 2, 10.0), (2000, 3, 100.0), (500, 4, 1.0)])
def test_fp64_converged_objective(gpulib, oracle, T, K, eps2):
    data, theta, x0, b, coeff = _qp(T, K, eps2, 7 * T + K, oracle)
    opts = dict(maxit=3000, stop_difff=0)
    xo, ro, _ = oracle.spgqp_solve(b, x0, T, K, coeff, oracle.spg_opts(**opts))
    with _problem(T, K, eps2, data, theta, x0, PASC_PREC_FP64) as p:
        st = p.spgqp_solve(capi.spgqp_opts(**opts))
        assert st.status in (capi.PASC_SPG_CONVERGED, capi.PASC_SPG_MAXIT, capi.PASC_SPG_DAD_ZERO)
        assert abs(st.fx - ro.fx) <= 1e-9 * abs(ro.fx)


@pytest.mark.parametrize("T,K,eps2", [(1000, 2, 10.0), (5000, 3, 100.0), (2000, 3, 1000.0),
                                      (800, 5, 5.0), (333, 8, 50.0), (4099, 1, 10.0)])
def test_mixed_converged_objective(gpulib, oracle, T, K, eps2):
    data, theta, x0, b, coeff = _qp(T, K, eps2, 11 * T + K, oracle)
    xo, ro, _ = oracle.spgqp_solve(b, x0, T, K, coeff, oracle.spg_opts(maxit=5000, eps=1e-13))
    with _problem(T, K, eps2, data, theta, x0, PASC_PREC_MIXED) as p:
        st = p.spgqp_solve(capi.spgqp_opts(maxit=3000, stop_difff=0))
        assert st.status != capi.PASC_SPG_NONFINITE
        assert abs(st.fx - ro.fx) <= 1e-6 * abs(ro.fx), (st.fx, ro.fx, st.it, st.status)
        g = p.get_gamma().reshape(T, K)
        assert np.all(g >= 0.0)
        assert np.max(np.abs(g.sum(axis=1) - 1.0)) <= 1e-5
        # the reported objective is the objective of the returned gamma
        f_host = 0.5 * g.ravel() @ oracle.matmult(g.ravel(), T, K, coeff) - b @ g.ravel()
        assert abs(f_host - st.fx) <= 1e-6 * abs(ro.fx)


def test_mixed_first_iterations_track_oracle(gpulib, oracle):
    T, K, eps2 = 4000, 3, 20.0
    data, theta, x0, b, coeff = _qp(T, K, eps2, 99, oracle)
    for maxit in (0, 1, 3, 10):
        _, ro, _ = oracle.spgqp_solve(b, x0.astype(np.float32).astype(np.float64), T, K, coeff,
                                      oracle.spg_opts(maxit=maxit))
        with _problem(T, K, eps2, data, theta, x0, PASC_PREC_MIXED) as p:
            st = p.spgqp_solve(capi.spgqp_opts(maxit=maxit))
            assert st.it == maxit and st.status == capi.PASC_SPG_MAXIT
            assert abs(st.fx - ro.fx) <= 2e-6 * abs(ro.fx), (maxit, st.fx, ro.fx)


def test_mixed_stop_rule_matches_reference_semantics(gpulib, oracle):
    """With the default |f - f_old| < eps test the GPU stops at an iteration where the
    objective change is below eps, and it counts hessmult as 1 + it."""
    T, K, eps2 = 3000, 3, 30.0
    data, theta, x0, b, coeff = _qp(T, K, eps2, 5, oracle)
    with _problem(T, K, eps2, data, theta, x0, PASC_PREC_MIXED) as p:
        st = p.spgqp_solve(capi.spgqp_opts(eps=1e-6, m=10))
        assert st.status == capi.PASC_SPG_CONVERGED
        assert st.hessmult == st.it + 1
        assert 0 < st.it < 1000


@pytest.mark.parametrize("prec", [PASC_PREC_FP64, PASC_PREC_MIXED])
def test_edge_sizes(gpulib, oracle, prec):
    """Small and tile-boundary sizes.  T == 1 has A = 0 (a linear program over one simplex):
    the reference divides by d'Ad = 0 there and ends at NaN or an infeasible point, so the
    check is against the analytic optimum -max_k b_k instead of the oracle."""
    for T, K in [(1, 1), (1, 4), (2, 2), (3, 3), (253, 3), (254, 2), (255, 2), (509, 7)]:
        data, theta, x0, b, coeff = _qp(T, K, 5.0, T * 13 + K, oracle)
        if T == 1:
            f_ref = -np.max(b)
        else:
            f_ref = oracle.spgqp_solve(b, x0, T, K, coeff, oracle.spg_opts(maxit=2000, eps=1e-13))[1].fx
        with _problem(T, K, 5.0, data, theta, x0, prec) as p:
            st = p.spgqp_solve(capi.spgqp_opts(maxit=2000, eps=1e-12))
            assert st.status != capi.PASC_SPG_NONFINITE
            tol = 1e-9 if prec == PASC_PREC_FP64 else 1e-6
            assert abs(st.fx - f_ref) <= tol * max(abs(f_ref), 1e-12), (T, K, st.fx, f_ref, st.status)
            g = p.get_gamma().reshape(T, K)
            assert np.all(g >= 0) and np.max(np.abs(g.sum(axis=1) - 1)) <= 1e-5


@pytest.mark.parametrize("prec", [PASC_PREC_FP64, PASC_PREC_MIXED])
def test_nonfinite_input_reports_status(gpulib, oracle, prec):
    """A NaN in the data makes b and the objective NaN: the solve stops with NONFINITE
    instead of iterating on garbage.  (A NaN in gamma does not propagate: the reference's
    projection maps such a block to zeros, and so does the GPU's.)"""
    T, K = 500, 2
    data, theta, x0, b, coeff = _qp(T, K, 5.0, 3, oracle)
    data = data.copy()
    data[10] = np.nan
    with _problem(T, K, 5.0, data, theta, x0, prec) as p:
        st = p.spgqp_solve(capi.spgqp_opts(maxit=50))
        assert st.status == capi.PASC_SPG_NONFINITE
    x0 = x0.copy()
    x0[10] = np.nan
    data, theta, _, b, coeff = _qp(T, K, 5.0, 3, oracle)
    xo, ro, _ = oracle.spgqp_solve(b, x0, T, K, coeff, oracle.spg_opts(maxit=20))
    with _problem(T, K, 5.0, data, theta, x0, prec) as p:
        st = p.spgqp_solve(capi.spgqp_opts(maxit=20))
        assert st.status == capi.PASC_SPG_MAXIT and np.isfinite(st.fx)
        tol = 1e-12 if prec == PASC_PREC_FP64 else 1e-5
        assert abs(st.fx - ro.fx) <= tol * abs(ro.fx)


def test_bad_arguments(gpulib):
    with pytest.raises(capi.PascError):
        Problem(0, 3)
    with pytest.raises(capi.PascError):
        Problem(100, 9, precision=PASC_PREC_MIXED)
    with pytest.raises(capi.PascError):
        Problem(100, 3, xdim=2, precision=PASC_PREC_FP64)  # multichannel data: mixed path only
    with pytest.raises(capi.PascError):
        Problem(100, 3, xdim=300)
    with Problem(10, 2) as p:
        with pytest.raises(capi.PascError):
            p.spgqp_solve(capi.spgqp_opts(m=0))
        with pytest.raises(capi.PascError):
            p.get_fx()
