"""The GPU adjoint (derivatives of a loss through the converged gamma-step QP) against the FP64
oracle's adjoint and against finite differences.

Tolerances: on an identical FP64 gamma the GPU's conjugate gradients differ from the oracle's
only in summation order: gradients within 1e-9 relative.  The mixed path hands the adjoint its
FP32 gamma (relative rounding 6e-8 on every entry) and solves in FP32 steps inside FP64
iterative refinement: gradients within 1e-5 relative.  Finite
differences (step 1e-4 relative) through tightly converged FP64 GPU solves agree to 1e-4."""
import numpy as np
import pytest

from pasc_inference_gb300 import PASC_PREC_FP64, PASC_PREC_MIXED, Problem, capi, datagen, learn

pytestmark = pytest.mark.gpu


def _signal(T, K, seed):
    levels = np.linspace(0.0, K - 1.0, K)
    return datagen.signal1d(T, K, levels, max(T // 40, 5), max(T // 8, 10), 0.4, seed)


def _converged(oracle, sig, theta, eps2):
    T, K = sig.T, sig.K
    b = oracle.residual_b(sig.data, theta, T, K)
    x, _, _ = oracle.spgqp_solve(b, oracle.project(sig.gamma0.copy(), T, K), T, K, oracle.A_coeff(eps2, T),
                                 oracle.spg_opts(m=10, eps=1e-14, maxit=20000))
    return x


def _rel(a, b):
    a, b = np.atleast_1d(a), np.atleast_1d(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("T,K,eps2", [(3000, 3, 20.0), (5000, 2, 100.0), (2000, 5, 10.0), (777, 8, 30.0)])
@pytest.mark.parametrize("prec", [PASC_PREC_FP64, PASC_PREC_MIXED])
def test_adjoint_matches_oracle_on_same_gamma(gpulib, oracle, T, K, eps2, prec):
    sig = _signal(T, K, T + K)
    theta = np.linspace(0.0, K - 1.0, K) + 0.03
    x = _converged(oracle, sig, theta, eps2)
    xin = x if prec == PASC_PREC_FP64 else x.astype(np.float32).astype(np.float64)
    loss_o, dg, dth_direct = oracle.recon_mse(xin, theta, sig.clean, T, K)
    # both conjugate-gradient solves to a relative residual of 1e-12, so that the comparison
    # measures the arithmetic rather than where each solve stopped
    deps_o, dX_o, dth_o, _, r_o = oracle.adjoint(xin, sig.data, theta, dg, T, K, eps2, cg_tol=1e-12)
    assert r_o.status == 1 and r_o.free_dims > 0
    with Problem(T, K, eps2, precision=prec) as p:
        p.set_data(sig.data)
        p.set_theta(theta)
        p.set_gamma(x)
        loss = p.recon_mse(sig.clean)
        deps, dX, dth, st = p.adjoint(opts=capi.adjoint_opts(cg_tol=1e-12))
        tol = 1e-9 if prec == PASC_PREC_FP64 else 1e-5
        assert abs(loss - loss_o) <= 1e-12 * loss_o
        assert st.status == 1 and st.free_dims == r_o.free_dims, (st.free_dims, r_o.free_dims)
        assert _rel(deps, deps_o) <= tol, (deps, deps_o)
        assert _rel(dX, dX_o) <= tol
        assert _rel(dth, dth_o + dth_direct) <= tol, (dth, dth_o + dth_direct)
        # an explicit dloss/dgamma gives the same result without the loss's own theta term
        deps2, dX2, dth2, _ = p.adjoint(dg, opts=capi.adjoint_opts(cg_tol=1e-12))
        assert _rel(deps2, deps) <= 1e-12 and _rel(dth2, dth_o) <= tol


def test_adjoint_end_to_end_mixed_vs_oracle(gpulib, oracle):
    """Solve on the GPU (mixed path, run to FP32 stagnation) and differentiate, against the
    oracle's FP64 solve (converged to ||d||^2 < 1e-28) and adjoint from the same inputs.  The
    gradient jumps where the free set changes: an oracle solve stopped at |f - f_old| < 1e-14
    (f within 2e-10 of the optimum) keeps one extra free entry and moves d loss/d epssqr by 1%,
    so both solves must reach the fixed point."""
    T, K, eps2 = 20000, 3, 50.0
    sig = _signal(T, K, 5)
    theta = np.array([0.0, 1.0, 2.0])
    b = oracle.residual_b(sig.data, theta, T, K)
    x, _, _ = oracle.spgqp_solve(b, oracle.project(sig.gamma0.copy(), T, K), T, K, oracle.A_coeff(eps2, T),
                                 oracle.spg_opts(m=10, eps=1e-28, maxit=60000, stop_difff=0, stop_normgp=1))
    _, dg, dth_direct = oracle.recon_mse(x, theta, sig.clean, T, K)
    deps_o, dX_o, dth_o, _, _ = oracle.adjoint(x, sig.data, theta, dg, T, K, eps2)
    with Problem(T, K, eps2, precision=PASC_PREC_MIXED) as p:
        p.set_data(sig.data)
        p.set_theta(theta)
        p.set_gamma(sig.gamma0)
        p.permute_gamma()
        p.update_b()
        p.spgqp_solve(capi.spgqp_opts(m=10, maxit=3000, stop_difff=0))
        p.recon_mse(sig.clean)
        deps, dX, dth, st = p.adjoint()
    assert _rel(deps, deps_o) <= 1e-4, (deps, deps_o)
    assert _rel(dth, dth_o + dth_direct) <= 1e-4
    assert np.corrcoef(dX, dX_o)[0, 1] >= 0.9999


def test_adjoint_finite_differences_fp64(gpulib, oracle):
    """Central differences (1e-4 relative) of the loss through FP64 GPU solves converged to
    ||d||^2 < 1e-26 and warm-started from the solution, against the GPU adjoint."""
    T, K, eps2 = 100000, 3, 30.0
    sig = _signal(T, K, 11)
    theta = np.array([0.0, 1.0, 2.0])
    opts = capi.spgqp_opts(m=10, eps=1e-26, maxit=30000, stop_difff=0, stop_normgp=1)
    with Problem(T, K, eps2, precision=PASC_PREC_FP64) as p:
        p.set_data(sig.data)
        p.set_theta(theta)
        p.set_gamma(sig.gamma0)
        p.permute_gamma()
        p.update_b()
        p.spgqp_solve(opts)
        x0 = p.get_gamma()
        p.recon_mse(sig.clean)
        deps, dX, dth, st = p.adjoint()
        h = 1e-4
        lo = []
        for e in (eps2 * (1 + h), eps2 * (1 - h)):
            p.set_epssqr(e)
            p.set_gamma(x0)
            p.update_b()
            p.spgqp_solve(opts)
            lo.append(p.recon_mse(sig.clean))
        fd = (lo[0] - lo[1]) / (2 * h * eps2)
        assert abs(fd - deps) <= 1e-4 * abs(deps), (fd, deps)
        p.set_epssqr(eps2)
        v = np.random.default_rng(1).normal(size=T)
        hx = 1e-4
        lo = []
        for sgn in (1, -1):
            p.set_data(sig.data + sgn * hx * v)
            p.set_gamma(x0)
            p.update_b()
            p.spgqp_solve(opts)
            lo.append(p.recon_mse(sig.clean))
        fd = (lo[0] - lo[1]) / (2 * hx)
        assert abs(fd - dX @ v) <= 1e-4 * np.abs(dX).sum(), (fd, dX @ v)


def test_descent_on_log_epssqr_lowers_the_loss(gpulib, oracle):
    """20 gradient steps on log epssqr from an over-regularised start: the loss falls, and the
    FP64 oracle's own solves agree that the end point is better than the start."""
    T, K = 20000, 3
    sig = _signal(T, K, 21)
    theta = np.array([0.0, 1.0, 2.0])
    with Problem(T, K, 3000.0, precision=PASC_PREC_MIXED) as p:
        p.set_data(sig.data)
        p.set_theta(theta)
        p.set_gamma(sig.gamma0)
        p.permute_gamma()
        rec = learn.descend_log_epssqr(p, sig.clean, steps=20)
    assert len(rec) == 21
    losses = [r["loss"] for r in rec]
    assert losses[-1] < 0.8 * losses[0], losses
    lo = [oracle.recon_mse(_converged(oracle, sig, theta, r["epssqr"]), theta, sig.clean, T, K)[0]
          for r in (rec[0], rec[-1])]
    assert lo[1] < 0.8 * lo[0], lo


def test_adjoint_errors(gpulib):
    with Problem(100, 3, 1.0) as p:
        with pytest.raises(capi.PascError):
            p.adjoint()  # no stored loss gradient
    with Problem(100, 9, 1.0, precision=PASC_PREC_FP64) as p:
        with pytest.raises(capi.PascError):
            p.recon_mse(np.zeros(100))  # K > 8
