"""TSSolver (theta step + SPG gamma step, outer loop) on the GPU against the reference-produced
golden runs and the FP64 oracle.

Acceptance (the path's stated accuracy): objective L within 1e-6 relative of FP64, theta
within 1e-5 relative, hard argmax labels equal on >= 99.99% of timesteps.  The fp64 path is
held to 1e-9 on L and 1e-7 on theta (its only difference from the reference is the order of
its dot-product sums)."""
import numpy as np
import pytest

from pasc_inference_gb300 import (PASC_PREC_FP64, PASC_PREC_MIXED, GraphH1FEMModel, Problem,
                                  Signal1DData, Decomposition, TSSolver, capi, datagen)

pytestmark = pytest.mark.gpu


def _golden_ts(golden):
    n = len({k.split("_")[1] for k in golden.files if k.startswith("ts_")})
    for i in range(n):
        T, K, eps2 = golden[f"ts_{i}_TKe"]
        yield (i, str(golden[f"ts_{i}_name"][0]), int(T), int(K), float(eps2))


def _run_ts(T, K, eps2, data, gamma0, prec, ts=None, spg=None):
    p = Problem(T, K, eps2, precision=prec)
    p.set_data(data)
    p.set_gamma(gamma0)
    p.set_theta(np.zeros(K))
    st = p.ts_solve(ts or capi.ts_opts(), spg or capi.spgqp_opts())
    return p, st


def _labels(g, T, K):
    return np.argmax(g.reshape(T, K), axis=1)


def _threl(th, ref):
    """theta error relative to the scale of theta: max_k |dtheta_k| / max_k |theta_k|."""
    return float(np.max(np.abs(th - ref)) / np.max(np.abs(ref)))


@pytest.mark.parametrize("prec", [PASC_PREC_FP64, PASC_PREC_MIXED])
def test_golden_tssolver_reference_settings(gpulib, golden, prec):
    """The reference's runs with its default settings (SPG stops on |f - f_old| < 1e-9, the
    outer loop on |L - L_old| < 1e-6 absolute).  Those rules stop short of the fixed point,
    and where they stop depends on rounding, so two correct implementations agree only to
    the accuracy the rules leave: L to 1e-4 relative, theta to 5e-3 of its scale, labels on
    >= 99.9% of timesteps (99.5% for the FP32-state path).  The tight comparison is test_tssolver_tight_vs_oracle."""
    for i, name, T, K, eps2 in _golden_ts(golden):
        L_ref = golden[f"ts_{i}_res"][0]
        th_ref, g_ref = golden[f"ts_{i}_theta"], golden[f"ts_{i}_gamma"]
        p, st = _run_ts(T, K, eps2, golden[f"ts_{i}_data"], golden[f"ts_{i}_gamma0"], prec)
        with p:
            th = p.get_theta()
            g = p.get_gamma()
        assert abs(st.L - L_ref) <= 1e-4 * abs(L_ref), (name, st.L, L_ref)
        assert _threl(th, th_ref) <= 5e-3, (name, th, th_ref)
        # the FP32-state path follows another trajectory and stops elsewhere short of the fixed
        # point: a few more ambiguous timesteps (gamma near 1/2) change their label
        agree = 0.999 if prec == PASC_PREC_FP64 else 0.995
        assert np.mean(_labels(g, T, K) == _labels(g_ref, T, K)) >= agree, name


TIGHT_CASES = [("k3_sigma05", dict(T=4000, K=3, levels=[0.0, 1.0, 2.0], smin=200, smax=800, sigma=0.5, seed=3), 20.0),
               ("k2_sigma08", dict(T=3000, K=2, levels=[1.0, 2.0], smin=200, smax=600, sigma=0.8, seed=21), 10.0),
               ("k3_eps300", dict(T=5000, K=3, levels=[0.0, 1.0, 2.0], smin=400, smax=1500, sigma=0.4, seed=11), 300.0),
               ("k4_sigma03", dict(T=5000, K=4, levels=[0.0, 1.0, 2.0, 3.0], smin=100, smax=500, sigma=0.3, seed=12), 5.0)]


@pytest.mark.parametrize("case", TIGHT_CASES, ids=[c[0] for c in TIGHT_CASES])
@pytest.mark.parametrize("prec", [PASC_PREC_FP64, PASC_PREC_MIXED])
def test_tssolver_tight_vs_oracle(gpulib, oracle, case, prec):
    """TSSolver driven to its fixed point (SPG |f - f_old| < 1e-13, outer |L - L_old| < 1e-13)
    on the GPU and in the FP64 oracle from identical inputs: L within 1e-6 relative (1e-9 for
    fp64), theta within 1e-5 of its scale, argmax labels equal on >= 99.99% of timesteps."""
    name, g, eps2 = case
    _tight_case(oracle, name, g, eps2, prec, tol_L=1e-9 if prec == PASC_PREC_FP64 else 1e-6,
                tol_th=1e-5, min_agree=0.9999)


@pytest.mark.parametrize("prec", [PASC_PREC_FP64, PASC_PREC_MIXED])
def test_tssolver_tight_ill_conditioned(gpulib, oracle, prec):
    """An ill-conditioned fixed point: with epssqr = 1000 over short segments two of the three
    clusters merge (theta_1 and theta_2 agree to 1e-4) and L is flat along the merge
    direction, so the fixed point moves with any rounding difference.  The FP64 GPU path
    still lands within 1e-8 of the oracle's L; the FP32-state path within 1e-5 on L and 1e-3
    on theta (measured 2e-6 / 2e-4), labels unchanged."""
    g = dict(T=3000, K=3, levels=[0.0, 1.0, 2.0], smin=100, smax=600, sigma=0.5, seed=7)
    if prec == PASC_PREC_FP64:
        _tight_case(oracle, "k3_eps1000_merged", g, 1000.0, prec, tol_L=1e-8, tol_th=1e-5, min_agree=0.9999)
    else:
        _tight_case(oracle, "k3_eps1000_merged", g, 1000.0, prec, tol_L=1e-5, tol_th=1e-3, min_agree=0.9999)


def _tight_case(oracle, name, g, eps2, prec, tol_L, tol_th, min_agree):
    sig = datagen.signal1d(g["T"], g["K"], g["levels"], g["smin"], g["smax"], g["sigma"], g["seed"])
    T, K = sig.T, sig.K
    g_o, th_o, r_o, _ = oracle.tssolver_solve(sig.data, sig.gamma0, np.zeros(K), T, K, eps2,
                                              ts=oracle.ts_opts(maxit=300, eps=1e-13),
                                              spg=oracle.spg_opts(m=10, eps=1e-13, maxit=20000))
    p, st = _run_ts(T, K, eps2, sig.data, sig.gamma0, prec, capi.ts_opts(maxit=300, eps=1e-13),
                    capi.spgqp_opts(m=10, eps=1e-13, maxit=20000))
    with p:
        th = p.get_theta()
        gam = p.get_gamma()
    assert abs(st.L - r_o.L) <= tol_L * abs(r_o.L), (name, st.L, r_o.L)
    assert _threl(th, th_o) <= tol_th, (name, th, th_o)
    assert np.mean(_labels(gam, T, K) == _labels(g_o, T, K)) >= min_agree, name


def test_mirror_classes_cfg0(gpulib, oracle):
    """The reference-style object graph (Decomposition, Signal1DData, GraphH1FEMModel, TSSolver)
    on the plain-method workload (T = 1e4, K = 2, levels {1, 2}, noise 1.0, epssqr 10), against
    the oracle's full TSSolver."""
    sig = datagen.signal1d_cfg0()
    T, K = sig.T, sig.K
    mydata = Signal1DData(sig.data)
    mydata.set_decomposition(Decomposition(T, 1, K, 1, 1))
    model = GraphH1FEMModel(mydata, 10.0, gamma0=sig.gamma0)
    solver = TSSolver(mydata, options={"spgqpsolver_m": 10, "spgqpsolver_eps": 1e-6})
    solver.solve()
    g_o, th_o, r_o, _ = oracle.tssolver_solve(sig.data, sig.gamma0, np.zeros(K), T, K, 10.0,
                                              spg=oracle.spg_opts(m=10, eps=1e-6))
    assert abs(solver.get_L() - r_o.L) <= 1e-6 * abs(r_o.L)
    th = mydata.get_thetavector()
    assert _threl(th, th_o) <= 1e-5
    agree = np.mean(_labels(mydata.get_gammavector(), T, K) == _labels(g_o, T, K))
    assert agree >= 0.9999
    # recovered signal error, as the driver reports it
    err = mydata.compute_abserr_reconstructed(sig.clean)
    err_o = oracle.abserr_reconstructed(g_o, th_o, sig.clean, T, K)
    assert abs(err - err_o) <= 1e-3 * err_o + 1e-6


def test_given_theta_and_relative_stop(gpulib, oracle):
    sig = datagen.signal1d(5000, 3, [0.0, 1.0, 2.0], 200, 800, 0.5, seed=11)
    T, K = sig.T, sig.K
    th0 = np.array([0.0, 1.0, 2.0])
    for prec in (PASC_PREC_FP64, PASC_PREC_MIXED):
        with Problem(T, K, 30.0, precision=prec) as p:
            p.set_data(sig.data)
            p.set_gamma(sig.gamma0)
            p.set_theta(th0)
            st = p.ts_solve(capi.ts_opts(thetasolved=1), capi.spgqp_opts(eps=1e-9))
            np.testing.assert_array_equal(p.get_theta(), th0)
            _, _, r, _ = oracle.tssolver_solve(sig.data, sig.gamma0, th0, T, K, 30.0,
                                               ts=oracle.ts_opts(thetasolved=1))
            assert abs(st.L - r.L) <= 1e-6 * abs(r.L)
        with Problem(T, K, 30.0, precision=prec) as p:
            p.set_data(sig.data)
            p.set_gamma(sig.gamma0)
            st = p.ts_solve(capi.ts_opts(relative=1, eps=1e-6), capi.spgqp_opts(eps=1e-9))
            _, _, r, _ = oracle.tssolver_solve(sig.data, sig.gamma0, np.zeros(K), T, K, 30.0,
                                               ts=oracle.ts_opts(relative=1, eps=1e-6))
            assert abs(st.L - r.L) <= 1e-6 * abs(r.L)


def test_annealing_keeps_best(gpulib, oracle):
    sig = datagen.signal1d(3000, 2, [1.0, 2.0], 200, 600, 0.8, seed=21)
    T, K = sig.T, sig.K
    restart = datagen.uniform(99, 0, T * K)
    with Problem(T, K, 10.0, precision=PASC_PREC_FP64) as p:
        p.set_data(sig.data)
        p.set_gamma(sig.gamma0)
        st = p.ts_solve(capi.ts_opts(annealing=3), capi.spgqp_opts(), gamma_restart=restart)
        _, _, r, _ = oracle.tssolver_solve(sig.data, sig.gamma0, np.zeros(K), T, K, 10.0,
                                           ts=oracle.ts_opts(annealing=3), gamma_restart=restart)
        assert abs(st.L - r.L) <= 1e-9 * abs(r.L)
        assert abs(st.aic - r.aic) <= 1e-9 * abs(r.aic) + 1e-12
        assert abs(st.it_sum - r.it_sum) <= 3
