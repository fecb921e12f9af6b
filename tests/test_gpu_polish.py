"""pasc_gb300_polish: FP64 face-Newton rounds from the end point of a solve to the optimum of
the gamma-step QP.

The mixed path's FP32 iteration stalls where its updates drop below half an FP32 ulp of gamma:
on ill-conditioned problems (large epssqr/T) that point lies 1e-6..1e-5 (relative 2-norm) from
the optimum and moves with the rounding of the sums.  After the polish the mixed gamma is the
optimum rounded to FP32: within 1e-6 of the FP64 optimum (measured ~1e-8), with the objective
within 1e-9 (the rounding moves f).  The reference optimum is the FP64 GPU solve driven to ||d||^2 < 1e-20 and then
polished itself; it is certified by its Frank-Wolfe gap under the oracle's operator and by the
oracle's own SPG iteration, which started there changes nothing."""
import numpy as np
import pytest

from pasc_inference_gb300 import PASC_PREC_FP64, PASC_PREC_MIXED, Problem, capi, datagen

pytestmark = pytest.mark.gpu

THETA = np.array([0.0, 1.0, 2.0])


def _load(sig, eps2, prec):
    p = Problem(sig.T, sig.K, eps2, precision=prec)
    p.set_data(sig.data)
    p.set_gamma(sig.gamma0)
    p.permute_gamma()
    p.set_theta(THETA)
    p.update_b()
    return p


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def sig():
    return datagen.signal1d_cfg1(T=200_000)


@pytest.fixture(scope="module")
def optima(sig, oracle):
    out = {}
    for eps2 in (100.0, 1000.0):
        with _load(sig, eps2, PASC_PREC_FP64) as p:
            p.spgqp_solve(capi.spgqp_opts(m=10, maxit=20000, eps=1e-20, stop_difff=0, stop_normgp=1))
            ps = p.polish()
            x = p.get_gamma()
        T, K = sig.T, sig.K
        coeff = oracle.A_coeff(eps2, T)
        b = oracle.residual_b(sig.data, THETA, T, K, nthreads=0)
        g = oracle.matmult(x, T, K, coeff, nthreads=0) - b
        f = 0.5 * (x @ (g + b)) - b @ x
        G, X = g.reshape(T, K), x.reshape(T, K)
        gap = float(np.sum(np.sum(X * G, axis=1) - G.min(axis=1)))
        assert gap <= 1e-12 * abs(f), (eps2, gap, f)
        assert abs(ps.fx - f) <= 1e-12 * abs(f), (eps2, ps.fx, f)
        xw, rw, _ = oracle.spgqp_solve(b, x, T, K, coeff, oracle.spg_opts(m=10, maxit=20, stop_difff=0), nthreads=0)
        assert abs(rw.fx - f) <= 1e-13 * abs(f) and _rel(xw, x) <= 1e-9, (eps2, rw.fx, f, _rel(xw, x))
        out[eps2] = (x, f)
    return out


@pytest.mark.parametrize("eps2", [100.0, 1000.0])
def test_polish_moves_mixed_fixed_point_onto_the_optimum(gpulib, sig, optima, eps2):
    xstar, fstar = optima[eps2]
    with _load(sig, eps2, PASC_PREC_MIXED) as p:
        p.spgqp_solve(capi.spgqp_opts(m=10, maxit=20000, stop_difff=0))
        before = _rel(p.get_gamma(), xstar)
        st = p.polish()
        xm = p.get_gamma()
        assert p.get_fx() == st.fx
    after = _rel(xm, xstar)
    assert st.rounds >= 1 and st.face_changes == 0, (st.rounds, st.face_changes)
    assert after <= 1e-6, (eps2, before, after)
    # the FP32 rounding of the polished gamma leaves sum_k gamma_tk off 1 by up to ~6e-8, which
    # moves f by up to ~1e-9 either way (measured 1.7e-10)
    assert abs(st.fx - fstar) <= 1e-9 * abs(fstar), (eps2, st.fx, fstar)
    assert np.all(xm >= 0.0)
    assert np.max(np.abs(xm.reshape(-1, 3).sum(axis=1) - 1.0)) <= 1e-6


def test_polish_shortens_the_fp64_solve(gpulib, sig, optima):
    """From 4000 FP64 iterations at epssqr 1000 (objective within 1e-8, gamma 5e-5 from the
    optimum) two or three rounds reach the optimum."""
    xstar, fstar = optima[1000.0]
    with _load(sig, 1000.0, PASC_PREC_FP64) as p:
        p.spgqp_solve(capi.spgqp_opts(m=10, maxit=4000, stop_difff=0))
        before = _rel(p.get_gamma(), xstar)
        st = p.polish(capi.polish_opts(rounds=8))
        after = _rel(p.get_gamma(), xstar)
    assert after <= 1e-9 and after < before, (before, after, st.rounds)


def test_polish_then_adjoint_matches_fp64(gpulib, sig):
    """The adjoint of the polished mixed solution agrees with the FP64 adjoint of the FP64
    optimum (the free sets and the A'gamma term now come from the same point)."""
    clean = datagen.signal1d_cfg1(T=200_000).clean
    eps2 = 300.0
    res = {}
    for prec in (PASC_PREC_MIXED, PASC_PREC_FP64):
        with _load(sig, eps2, prec) as p:
            if prec == PASC_PREC_MIXED:
                p.spgqp_solve(capi.spgqp_opts(m=10, maxit=20000, stop_difff=0))
            else:
                p.spgqp_solve(capi.spgqp_opts(m=10, maxit=20000, eps=1e-20, stop_difff=0, stop_normgp=1))
            p.polish()
            p.recon_mse(clean)
            d, _, _, _ = p.adjoint()
            res[prec] = d
    rel = abs(res[PASC_PREC_MIXED] - res[PASC_PREC_FP64]) / abs(res[PASC_PREC_FP64])
    assert rel <= 1e-5, (res, rel)


def test_polish_restrictions(gpulib):
    with Problem(100, 3, 1.0, precision=PASC_PREC_MIXED) as p:
        with pytest.raises(capi.PascError):
            p.polish(capi.polish_opts(rounds=-1))
    with Problem(100, 3, 1.0, precision=PASC_PREC_MIXED, xdim=4) as p:
        with pytest.raises(capi.PascError):
            p.polish()
