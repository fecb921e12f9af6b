"""SPGQPSolverC (GraphH1FEMModel gammasolvertype 2: the coefficient of A factored out of the
SPG iteration) on the GPU against the oracle's restatement of spgqpsolver_coeff.h:611-835.

- fp64 path: a fixed-length run follows the oracle's iterates (f within 1e-11 relative, gamma
  within 1e-9); converged runs within 1e-9;
- mixed path (both 1-D sweep kernels and the graph sweep): converged objective within 1e-6
  (1e-5 on the stiff epssqr = 3000 case);
- TSSolver with the coefficient solver, 1-D and image: fp64 L within 1e-9, mixed within 1e-6;
- solver types 3 and 4 (PERMON, TAO) and the combination with theta in the penalty are
  refused."""
import numpy as np
import pytest

from pasc_inference_gb300 import (PASC_PREC_FP64, PASC_PREC_MIXED, BGMGraphGrid2D, PascError, Problem, capi,
                                  datagen)

pytestmark = pytest.mark.gpu


def test_types(gpulib):
    with Problem(100, 3, 1.0) as p:
        assert p.get_gamma_solver_type() == 1
        p.set_gamma_solver_type(2)
        assert p.get_gamma_solver_type() == 2
        p.set_gamma_solver_type(0)
        assert p.get_gamma_solver_type() == 1
        for t in (3, 4):
            with pytest.raises(PascError) as e:
                p.set_gamma_solver_type(t)
            assert e.value.code == capi.PASC_ERR_NOTSUPP
        p.set_usethetainpenalty(True)
        with pytest.raises(PascError) as e:
            p.set_gamma_solver_type(2)
        assert e.value.code == capi.PASC_ERR_NOTSUPP


CASES = [(PASC_PREC_FP64, None), (PASC_PREC_MIXED, 0), (PASC_PREC_MIXED, 1)]


@pytest.mark.parametrize("prec,variant", CASES)
@pytest.mark.parametrize("eps2", [30.0, 3000.0])
def test_spgqp_coeff_vs_oracle(gpulib, oracle, prec, variant, eps2):
    T, K = 5000, 3
    sig = datagen.signal1d(T, K, [0.0, 1.0, 2.0], 100, 500, 0.5, 4)
    theta = np.array([0.0, 1.0, 2.0])
    b = oracle.residual_b(sig.data, theta, T, K)
    x0 = datagen.normalised_gamma(sig.gamma0, T, K)
    coeff = oracle.A_coeff(eps2, T)
    fp64 = prec == PASC_PREC_FP64
    runs = [(dict(maxit=50, eps=0.0, m=10), 1e-11)] if fp64 else []
    # epssqr = 3000 over T = 5000 is the stiff case (A = 0.6 A_hat against b ~ 1e-4): the FP32
    # state resolves its objective to ~3e-6 (as for SPGQPSolver on ill-conditioned fixed points)
    runs.append((dict(maxit=50000, eps=1e-13, m=10), 1e-9 if fp64 else (1e-6 if eps2 < 1000 else 1e-5)))
    for opts, tol in runs:
        x_o, r_o = oracle.spgqp_solve_coeff(b, x0, T, K, coeff, oracle.spg_opts(**opts))
        with Problem(T, K, eps2, precision=prec) as p:
            if variant is not None:
                p.set_sweep_variant(variant)
            p.set_gamma_solver_type(2)
            p.set_data(sig.data)
            p.set_gamma(x0)
            p.set_theta(theta)
            p.update_b()
            st = p.spgqp_solve(capi.spgqp_opts(**opts))
            x = p.get_gamma()
        assert abs(st.fx - r_o.fx) <= tol * abs(r_o.fx), (opts, st.fx, r_o.fx)
        if opts["eps"] == 0.0:
            assert st.it == r_o.it and np.max(np.abs(x - x_o)) <= 1e-9


@pytest.mark.parametrize("prec", [PASC_PREC_FP64, PASC_PREC_MIXED])
def test_tssolver_coeff_vs_oracle(gpulib, oracle, prec):
    sig = datagen.signal1d(4000, 3, [0.0, 1.0, 2.0], 200, 800, 0.5, 3)
    T, K = sig.T, sig.K
    ts_kw = dict(maxit=300, eps=1e-13)
    spg_kw = dict(m=10, eps=1e-13, maxit=20000)
    g_o, th_o, r_o = oracle.tssolver_solve_coeff(sig.data, sig.gamma0, np.zeros(K), T, K, 20.0,
                                                 ts=oracle.ts_opts(**ts_kw), spg=oracle.spg_opts(**spg_kw))
    with Problem(T, K, 20.0, precision=prec) as p:
        p.set_gamma_solver_type(2)
        p.set_data(sig.data)
        p.set_gamma(sig.gamma0)
        p.set_theta(np.zeros(K))
        st = p.ts_solve(capi.ts_opts(**ts_kw), capi.spgqp_opts(**spg_kw))
        th = p.get_theta()
    tol_L, tol_th = (1e-9, 1e-7) if prec == PASC_PREC_FP64 else (1e-6, 1e-5)
    assert abs(st.L - r_o.L) <= tol_L * abs(r_o.L)
    assert np.max(np.abs(th - th_o)) <= tol_th * np.max(np.abs(th_o))


@pytest.mark.parametrize("prec", [PASC_PREC_FP64, PASC_PREC_MIXED])
def test_image_coeff_vs_oracle(gpulib, oracle, prec):
    w, h, K = 48, 40, 2
    rng = np.random.default_rng(2)
    yy, xx = np.mgrid[0:h, 0:w]
    data = ((((xx - w / 3) ** 2 + (yy - h / 2) ** 2) < (h / 4) ** 2).astype(float).ravel()
            + 0.4 * rng.standard_normal(w * h))
    g = BGMGraphGrid2D(w, h)
    g.process_grid()
    g0 = datagen.uniform(5, 0, w * h * K)
    ts_kw = dict(maxit=300, eps=1e-13)
    spg_kw = dict(m=10, eps=1e-13, maxit=20000)
    g_o, th_o, r_o = oracle.tssolver_solve_coeff(data, g0, np.zeros(K), 1, K, 1.5, g.ptr, g.idx,
                                                 ts=oracle.ts_opts(**ts_kw), spg=oracle.spg_opts(**spg_kw))
    with Problem(1, K, 1.5, precision=prec, graph=g) as p:
        p.set_gamma_solver_type(2)
        p.set_data(data)
        p.set_gamma(g0)
        p.set_theta(np.zeros(K))
        st = p.ts_solve(capi.ts_opts(**ts_kw), capi.spgqp_opts(**spg_kw))
    tol_L = 1e-9 if prec == PASC_PREC_FP64 else 1e-6
    assert abs(st.L - r_o.L) <= tol_L * abs(r_o.L)
