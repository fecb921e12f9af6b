"""Theta in the penalty (GraphH1FEMModel with usethetainpenalty) on the GPU against the FP64
oracle.

- theta step: fp64 within 1e-12 relative (the sums are taken in another order); mixed within
  1e-5 relative (FP32 gamma and data, FP64 partial sums);
- block-scaled gamma QP at a fixed theta: a fixed-length run follows the oracle's iterates
  (fp64 f within 1e-11 relative, mixed within 1e-6);
- TSSolver at its fixed point: fp64 L within 1e-8 relative and theta within 1e-6 of its
  scale; mixed L within 1e-6 and theta within 1e-5; labels agree on >= 99.9% of timesteps;
- the cases the reference cannot run (multichannel data, FEM reduction) and the adjoint are
  refused with PASC_ERR_NOTSUPP."""
import numpy as np
import pytest

from pasc_inference_gb300 import (PASC_PREC_FP64, PASC_PREC_MIXED, Decomposition, Fem, GraphH1FEMModel, PascError,
                                  Problem, Signal1DData, TSSolver, capi, datagen)

pytestmark = pytest.mark.gpu


def _sig(T=4000, K=3, seed=3):
    return datagen.signal1d(T, K, [0.0, 1.0, 2.0][:K] if K <= 3 else list(np.linspace(0, 2, K)), 200, 800, 0.5,
                            seed)


def test_refusals(gpulib):
    with Problem(1000, 3, 10.0, precision=PASC_PREC_MIXED, xdim=4) as p:
        with pytest.raises(PascError) as e:
            p.set_usethetainpenalty(True)
        assert e.value.code == capi.PASC_ERR_NOTSUPP
    with Problem(1000, 3, 10.0) as p:
        p.set_fem(0.5, 0)
        with pytest.raises(PascError) as e:
            p.set_usethetainpenalty(True)
        assert e.value.code == capi.PASC_ERR_NOTSUPP
    with Problem(1000, 3, 10.0) as p:
        p.set_usethetainpenalty(True)
        assert p.get_usethetainpenalty()
        with pytest.raises(PascError) as e:
            p.set_fem(0.5, 0)
        assert e.value.code == capi.PASC_ERR_NOTSUPP
        p.set_fem(1.0, 0)  # no reduction: fine
        p.set_usethetainpenalty(False)
        assert not p.get_usethetainpenalty()
    sig = _sig(2000)
    with Problem(sig.T, sig.K, 10.0, precision=PASC_PREC_FP64) as p:
        p.set_usethetainpenalty(True)
        p.set_data(sig.data)
        p.set_gamma(sig.gamma0)
        p.set_theta(np.array([0.1, 1.0, 1.9]))
        p.update_b()
        p.spgqp_solve(capi.spgqp_opts(maxit=50))
        with pytest.raises(PascError) as e:
            p.adjoint(np.zeros(sig.T * sig.K))
        assert e.value.code == capi.PASC_ERR_NOTSUPP


@pytest.mark.parametrize("prec", [PASC_PREC_FP64, PASC_PREC_MIXED])
@pytest.mark.parametrize("T,K", [(1, 2), (7, 3), (5000, 3), (100003, 5)])
def test_theta_step(gpulib, oracle, prec, T, K):
    rng = np.random.default_rng(T + K)
    g = oracle.project(rng.random(T * K), T, K)
    data = rng.standard_normal(T)
    eps2 = 50.0
    with Problem(T, K, eps2, precision=prec) as p:
        p.set_usethetainpenalty(True)
        p.set_data(data)
        p.set_gamma(g)
        p.update_theta()
        th = p.get_theta()
    alpha = oracle.A_coeff(eps2, T)
    if prec == PASC_PREC_FP64:
        ref = oracle.theta_update_penalty(g, data, T, K, alpha)
        np.testing.assert_allclose(th, ref, rtol=1e-12, atol=1e-14)
    else:
        g32 = g.astype(np.float32).astype(np.float64)
        d32 = data.astype(np.float32).astype(np.float64)
        ref = oracle.theta_update_penalty(g32, d32, T, K, alpha)
        np.testing.assert_allclose(th, ref, rtol=1e-5, atol=1e-6 * np.max(np.abs(ref)))


@pytest.mark.parametrize("prec,variant", [(PASC_PREC_FP64, None), (PASC_PREC_MIXED, 0), (PASC_PREC_MIXED, 1)])
def test_gamma_qp_fixed_theta(gpulib, oracle, prec, variant):
    """A fixed-length run (no stopping test) follows the oracle's iterates: fp64 50 iterations,
    f within 1e-11 relative and gamma within 1e-9; mixed 10 iterations, f within 1e-5 and
    gamma within 1e-4 (FP32 rounding enters every iteration: 5e-6 after 20).  The converged runs (|f - f_old| < 1e-13) stop at nearby iterations: f
    within 1e-8 (fp64) or 1e-6 (mixed), labels on >= 99.9% of timesteps.  With theta_0 = 0.05
    this QP is ill-conditioned and the BB steps amplify rounding: in the oracle alone a 1-ulp
    change of the coefficients moves f by 2e-13 after 50 iterations, 1.5e-2 after 300, and
    2e-9 at the converged stop; a 1e-7 change (FP32) moves f by 6e-8 after 20 iterations."""
    sig = _sig(6000, 3, 5)
    T, K = sig.T, sig.K
    theta = np.array([0.05, 0.9, 2.1])
    eps2 = 200.0
    alpha = oracle.A_coeff(eps2, T)
    kc = np.array([alpha * theta[k] * theta[k] for k in range(K)])
    x0 = datagen.normalised_gamma(sig.gamma0, T, K)
    b = oracle.residual_b(sig.data, theta, T, K)
    fp64 = prec == PASC_PREC_FP64
    for opts, tol_f, tol_x in ((dict(maxit=50 if fp64 else 10, eps=0.0, m=10), 1e-11 if fp64 else 1e-5,
                                1e-9 if fp64 else 1e-4),
                               (dict(maxit=20000, eps=1e-13, m=10), 1e-8 if fp64 else 1e-6, None)):
        x_o, r_o = oracle.spgqp_solve_kc(b, x0, T, K, kc, oracle.spg_opts(**opts))
        with Problem(T, K, eps2, precision=prec) as p:
            if variant is not None:
                p.set_sweep_variant(variant)
            p.set_usethetainpenalty(True)
            p.set_data(sig.data)
            p.set_gamma(x0)
            p.set_theta(theta)
            p.update_b()
            st = p.spgqp_solve(capi.spgqp_opts(**opts))
            x = p.get_gamma()
        assert abs(st.fx - r_o.fx) <= tol_f * abs(r_o.fx), (opts, st.fx, r_o.fx)
        if tol_x is not None:
            assert st.it == r_o.it
            assert np.max(np.abs(x - x_o)) <= tol_x
        lab, lab_o = np.argmax(x.reshape(T, K), axis=1), np.argmax(x_o.reshape(T, K), axis=1)
        assert np.mean(lab == lab_o) >= 0.999


def test_uniform_theta_equals_plain(gpulib):
    """Theta = 1 in every cluster: the weighted sweep solves the unweighted QP (the weighted
    kernel may run on another grid, so the partial sums are added in another order)."""
    sig = _sig(5000, 3, 9)
    T, K = sig.T, sig.K
    out = []
    for tp in (False, True):
        with Problem(T, K, 30.0) as p:
            p.set_sweep_variant(1)
            if tp:
                p.set_usethetainpenalty(True)
            p.set_data(sig.data)
            p.set_gamma(datagen.normalised_gamma(sig.gamma0, T, K))
            p.set_theta(np.ones(K))
            p.update_b()
            st = p.spgqp_solve(capi.spgqp_opts(maxit=300, eps=0.0))
            out.append((st.fx, p.get_gamma()))
    assert abs(out[0][0] - out[1][0]) <= 1e-6 * abs(out[0][0])
    np.testing.assert_allclose(out[0][1], out[1][1], atol=1e-4)


@pytest.mark.parametrize("eps2", [1.0, 100.0])
@pytest.mark.parametrize("prec,variant", [(PASC_PREC_FP64, None), (PASC_PREC_MIXED, 0), (PASC_PREC_MIXED, 1)])
def test_tssolver_vs_oracle(gpulib, oracle, eps2, prec, variant):
    sig = _sig(4000, 3, 3)
    T, K = sig.T, sig.K
    ts_kw = dict(maxit=300, eps=1e-13)
    spg_kw = dict(m=10, eps=1e-13, maxit=20000)
    g_o, th_o, r_o = oracle.tssolver_solve_model(sig.data, sig.gamma0, np.zeros(K), T, K, eps2,
                                                 usethetainpenalty=True, ts=oracle.ts_opts(**ts_kw),
                                                 spg=oracle.spg_opts(**spg_kw))
    with Problem(T, K, eps2, precision=prec) as p:
        if variant is not None:
            p.set_sweep_variant(variant)
        p.set_usethetainpenalty(True)
        p.set_data(sig.data)
        p.set_gamma(sig.gamma0)
        p.set_theta(np.zeros(K))
        st = p.ts_solve(capi.ts_opts(**ts_kw), capi.spgqp_opts(**spg_kw))
        th = p.get_theta()
        gam = p.get_gamma()
    # (the inner solves stop at |f - f_old| < 1e-13, where this QP family is resolved to ~2e-9
    # relative: see test_gamma_qp_fixed_theta)
    tol_L, tol_th = (1e-8, 1e-6) if prec == PASC_PREC_FP64 else (1e-6, 1e-5)
    assert abs(st.L - r_o.L) <= tol_L * abs(r_o.L), (st.L, r_o.L)
    assert np.max(np.abs(th - th_o)) <= tol_th * np.max(np.abs(th_o)), (th, th_o)
    lab, lab_o = np.argmax(gam.reshape(T, K), axis=1), np.argmax(g_o.reshape(T, K), axis=1)
    assert np.mean(lab == lab_o) >= 0.999


def test_model_class_surface(gpulib, oracle):
    sig = _sig(3000, 3, 21)
    data = Signal1DData(sig.data)
    data.set_decomposition(Decomposition(sig.T, 1, sig.K, 1, 1))
    model = GraphH1FEMModel(data, 10.0, usethetainpenalty=True, precision=PASC_PREC_FP64, gamma0=sig.gamma0)
    assert model.get_usethetainpenalty() and model.problem.get_usethetainpenalty()
    solver = TSSolver(data, options={"tssolver_maxit": 200, "tssolver_eps": 1e-12, "spgqpsolver_eps": 1e-13,
                                     "spgqpsolver_maxit": 20000})
    solver.solve()
    g_o, th_o, r_o = oracle.tssolver_solve_model(sig.data, sig.gamma0, np.zeros(sig.K), sig.T, sig.K, 10.0,
                                                 usethetainpenalty=True,
                                                 ts=oracle.ts_opts(maxit=200, eps=1e-12),
                                                 spg=oracle.spg_opts(eps=1e-13, maxit=20000))
    assert abs(solver.get_L() - r_o.L) <= 1e-8 * abs(r_o.L)
    data2 = Signal1DData(sig.data)
    data2.set_decomposition(Decomposition(sig.T, 1, sig.K, 1, 1))
    with pytest.raises(PascError):
        GraphH1FEMModel(data2, 10.0, fem=Fem(0.5), usethetainpenalty=True)
