"""The reference's OWN generic solvers on GPU vectors: SPGQPSolver<GB300Vec>::solve and
TSSolver<GB300Vec>::solve (include/general/solver/spgqpsolver.h:575-805, tssolver.h:492-715),
compiled unmodified from the PASC_inference headers with the GB300 backend of
include/pasc/gb300_backend.hpp, every vector operation a C-ABI call on the device
(tests/cpp/gb300_backend_driver.cpp; oracle/build_ref.sh writes it out as one translation
unit with the reference's headers inlined, which is compiled here).  Skipped where that file
was not made (no reference tree when the repository was prepared).

Against the FP64 oracle (the restatement pinned bit for bit to the same templates on host
arrays): the backend runs the same FP64 operations, only its dot products are summed in a
block tree, so fixed-length SPG runs agree to 1e-11 on the objective and the TSSolver fixed
point to 1e-9 (L) and 1e-8 (theta); and against the library's own FP64 path
(pasc_gb300_ts_solve), the same fixed point to 1e-9."""
import os
import struct
import subprocess

import numpy as np
import pytest

from pasc_inference_gb300 import PASC_PREC_FP64, Problem, capi, datagen
from pasc_inference_gb300 import build as B

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FLAT = os.path.join(ROOT, "oracle", "_ref", "backend", "gb300_backend_driver_flat.cpp")
EXE = os.path.join(ROOT, "tests", "cpp", "_build", "gb300_backend_driver")


@pytest.fixture(scope="module")
def driver(gpulib):
    if not os.path.exists(FLAT):
        pytest.skip("oracle/_ref/backend not made (oracle/build_ref.sh found no reference tree)")
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    if not os.path.exists(EXE) or os.path.getmtime(EXE) < max(os.path.getmtime(FLAT), os.path.getmtime(B.LIB_PATH)):
        subprocess.check_call(["g++", "-std=c++14", "-O2", "-w", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                               FLAT, "-L", B.PKG, "-lpasc_gb300", "-Wl,-rpath," + B.PKG, "-o", EXE])
    return EXE


def _run(exe, tmp_path, mode, data, theta, gamma, K, eps2, spg_maxit, spg_eps, stop_difff=1, ts_maxit=300,
         ts_eps=1e-6, m=10):
    T = len(data)
    fin, fout = tmp_path / f"in{mode}.bin", tmp_path / f"out{mode}.bin"
    with open(fin, "wb") as f:
        f.write(struct.pack("3i", mode, T, K))
        f.write(np.array([eps2, spg_maxit, spg_eps, m, stop_difff, ts_maxit, ts_eps], dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(data, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(theta, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(gamma, dtype=np.float64).tobytes())
    r = subprocess.run([exe, str(fin), str(fout)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = np.fromfile(fout, dtype=np.float64)
    return out[0], int(out[1]), int(out[2]), out[3:3 + K], out[3 + K:]


@pytest.mark.parametrize("T,K,eps2", [(5000, 3, 20.0), (3001, 2, 100.0), (2000, 5, 5.0)])
def test_reference_spgqp_on_gpu_vectors(driver, oracle, tmp_path, T, K, eps2):
    rng = np.random.default_rng(T + K)
    data = rng.normal(size=T) * 0.5 + rng.integers(0, K, size=T)
    theta = np.arange(K, dtype=float)
    x0 = rng.random(T * K)
    b = oracle.residual_b(data, theta, T, K)
    coeff = oracle.A_coeff(eps2, T)
    for maxit in (1, 5, 20):
        fx, it, hm, _, g = _run(driver, tmp_path, 0, data, theta, x0, K, eps2, maxit, 0.0, stop_difff=0)
        xo, ro, _ = oracle.spgqp_solve(b, x0, T, K, coeff, oracle.spg_opts(maxit=maxit, m=10, stop_difff=0))
        assert it == ro.it == maxit and hm == ro.hessmult
        assert abs(fx - ro.fx) <= 1e-11 * abs(ro.fx), (maxit, fx, ro.fx)
        np.testing.assert_allclose(g, xo, rtol=0, atol=1e-9)


def test_reference_tssolver_on_gpu_vectors(driver, oracle, tmp_path):
    sig = datagen.signal1d(4000, 3, [0.0, 1.0, 2.0], 200, 800, 0.5, 3)
    T, K, eps2 = sig.T, sig.K, 20.0
    L, it, it_sum, th, g = _run(driver, tmp_path, 1, sig.data, np.zeros(K), sig.gamma0, K, eps2, 20000, 1e-13,
                                ts_maxit=300, ts_eps=1e-13)
    g_o, th_o, r_o, _ = oracle.tssolver_solve(sig.data, sig.gamma0, np.zeros(K), T, K, eps2,
                                              ts=oracle.ts_opts(maxit=300, eps=1e-13),
                                              spg=oracle.spg_opts(m=10, eps=1e-13, maxit=20000))
    assert abs(L - r_o.L) <= 1e-9 * abs(r_o.L), (L, r_o.L)
    assert np.max(np.abs(th - th_o)) <= 1e-8 * np.max(np.abs(th_o)), (th, th_o)
    assert np.mean(np.argmax(g.reshape(T, K), 1) == np.argmax(g_o.reshape(T, K), 1)) >= 0.9999
    with Problem(T, K, eps2, precision=PASC_PREC_FP64) as p:
        p.set_data(sig.data)
        p.set_gamma(sig.gamma0)
        p.set_theta(np.zeros(K))
        st = p.ts_solve(capi.ts_opts(maxit=300, eps=1e-13), capi.spgqp_opts(m=10, eps=1e-13, maxit=20000))
    assert abs(L - st.L) <= 1e-9 * abs(st.L), (L, st.L)
