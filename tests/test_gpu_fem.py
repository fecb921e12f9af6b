"""FEM temporal coarsening on the GPU against the FP64 oracle: the reduce / prolongate entry
points (bit-identical: same FP64 operations in the same order), and the reduced TSSolver
(GraphH1FEMModel with fem_reduce < 1) of both precisions at its fixed point: fp64 L within
1e-9 relative and theta within 1e-7 of its scale (the SPG dot products are summed in another
order); mixed L within 1e-6 and theta within 1e-5."""
import ctypes as C

import numpy as np
import pytest

from pasc_inference_gb300 import (PASC_PREC_FP64, PASC_PREC_MIXED, Decomposition, Fem, FemHat,
                                  GraphH1FEMModel, Problem, Signal1DData, TSSolver, capi, datagen)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


@pytest.mark.parametrize("fem_type", [0, 1])
@pytest.mark.parametrize("T1,r,K", [(5, 0.4, 1), (1001, 0.5, 3), (4096, 0.1, 2), (777, 0.9, 4), (100000, 0.33, 3)])
def test_reduce_prolongate_bit_exact(gpulib, torch_cuda, oracle, fem_type, T1, r, K):
    torch = torch_cuda
    T2 = oracle.fem_T_reduced(T1, r)
    rng = np.random.default_rng(T1 + K)
    g1 = rng.random(T1 * K)
    g2 = rng.random(T2 * K)
    d1 = torch.tensor(g1, dtype=torch.float64, device="cuda")
    d2 = torch.empty(T2 * K, dtype=torch.float64, device="cuda")
    assert gpulib.pasc_gb300_fem_reduce_f64(C.c_void_p(d1.data_ptr()), C.c_void_p(d2.data_ptr()), T1, T2, K,
                                            fem_type, None) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d2.cpu().numpy(), oracle.fem_reduce(g1, T1, T2, K, fem_type))
    e2 = torch.tensor(g2, dtype=torch.float64, device="cuda")
    e1 = torch.zeros(T1 * K, dtype=torch.float64, device="cuda")
    assert gpulib.pasc_gb300_fem_prolongate_f64(C.c_void_p(e2.data_ptr()), C.c_void_p(e1.data_ptr()), T1, T2, K,
                                                fem_type, None) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(e1.cpu().numpy(), oracle.fem_prolongate(g2, T1, T2, K, fem_type))


CASES = [("sum_half", dict(T=4000, K=3, levels=[0.0, 1.0, 2.0], smin=200, smax=800, sigma=0.5, seed=3), 20.0, 0.5, 0),
         ("sum_tenth", dict(T=6000, K=2, levels=[1.0, 2.0], smin=300, smax=900, sigma=0.6, seed=8), 10.0, 0.1, 0),
         ("hat_third", dict(T=5000, K=3, levels=[0.0, 1.0, 2.0], smin=300, smax=1000, sigma=0.4, seed=11), 30.0, 0.33, 1)]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("prec", [PASC_PREC_FP64, PASC_PREC_MIXED])
def test_reduced_tssolver_vs_oracle(gpulib, oracle, case, prec):
    name, g, eps2, r, fem_type = case
    sig = datagen.signal1d(g["T"], g["K"], g["levels"], g["smin"], g["smax"], g["sigma"], g["seed"])
    T, K = sig.T, sig.K
    ts_kw = dict(maxit=300, eps=1e-13)
    spg_kw = dict(m=10, eps=1e-13, maxit=20000)
    g_o, th_o, r_o = oracle.tssolver_solve_fem(sig.data, sig.gamma0, np.zeros(K), T, K, eps2, r, fem_type,
                                               ts=oracle.ts_opts(**ts_kw), spg=oracle.spg_opts(**spg_kw))
    with Problem(T, K, eps2, precision=prec) as p:
        p.set_fem(r, fem_type)
        assert p.get_fem()[2] == oracle.fem_T_reduced(T, r)
        p.set_data(sig.data)
        p.set_gamma(sig.gamma0)
        p.set_theta(np.zeros(K))
        st = p.ts_solve(capi.ts_opts(**ts_kw), capi.spgqp_opts(**spg_kw))
        th = p.get_theta()
        gam = p.get_gamma()
        assert p.get_fx() == st.L
    tol_L, tol_th = (1e-9, 1e-7) if prec == PASC_PREC_FP64 else (1e-6, 1e-5)
    assert abs(st.L - r_o.L) <= tol_L * abs(r_o.L), (name, st.L, r_o.L)
    assert np.max(np.abs(th - th_o)) <= tol_th * np.max(np.abs(th_o)), (name, th, th_o)
    lab, lab_o = np.argmax(gam.reshape(T, K), axis=1), np.argmax(g_o.reshape(T, K), axis=1)
    assert np.mean(lab == lab_o) >= 0.999, name


def test_unreduced_limit(gpulib):
    sig = datagen.signal1d(3000, 3, [0.0, 1.0, 2.0], 200, 600, 0.5, 3)
    res = []
    for fem in (None, 1.0):
        with Problem(3000, 3, 20.0, precision=PASC_PREC_FP64) as p:
            if fem is not None:
                p.set_fem(fem, 0)
            p.set_data(sig.data)
            p.set_gamma(sig.gamma0)
            p.set_theta(np.zeros(3))
            res.append((p.ts_solve().L, p.get_theta()))
    assert res[0][0] == res[1][0] and np.array_equal(res[0][1], res[1][1])


def test_mirror_classes_with_fem(gpulib, oracle):
    sig = datagen.signal1d(4000, 3, [0.0, 1.0, 2.0], 200, 800, 0.5, 4)
    for fem in (Fem(0.25), FemHat(0.25)):
        data = Signal1DData(sig.data)
        data.set_decomposition(Decomposition(4000, 1, 3, 1, 1))
        GraphH1FEMModel(data, 20.0, fem=fem, gamma0=sig.gamma0)
        solver = TSSolver(data, options={"spgqpsolver_m": 10})
        solver.solve()
        _, th_o, r_o = oracle.tssolver_solve_fem(sig.data, sig.gamma0, np.zeros(3), 4000, 3, 20.0, 0.25,
                                                 fem.fem_type, spg=oracle.spg_opts(m=10))
        assert np.isfinite(solver.get_L())
        assert abs(solver.get_L() - r_o.L) <= 1e-3 * abs(r_o.L)  # reference stopping rules: loose


def test_fem_argument_errors(gpulib):
    with Problem(100, 3, 1.0) as p:
        for bad in ((0.0, 0), (1.5, 0), (0.5, 2)):
            with pytest.raises(capi.PascError):
                p.set_fem(*bad)
        p.set_fem(0.5, 0)
        with pytest.raises(capi.PascError):
            p.spgqp_start(capi.spgqp_opts())
        with pytest.raises(capi.PascError):
            p.recon_mse(np.zeros(100))
    with Problem(3, 2, 1.0) as p:
        with pytest.raises(capi.PascError):
            p.set_fem(0.3, 1)  # FEM-HAT needs two coarse points
