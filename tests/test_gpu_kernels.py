"""GPU kernels through the C ABI against the FP64 oracle: simplex projection and the FEM-H1
operator, both precisions.  Device buffers come from torch (test plumbing only).

Tolerances: fp64 forms are bit-identical to the oracle (same operation order, no FMA);
fp32 forms are compared with the oracle run on the FP32-rounded input, |diff| <= 2e-6 for
projections (values in [0, 1]) and relative 1e-6 of max|y| for the operator."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


def _dev(torch, a, dtype):
    return torch.tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _proj_cases(golden):
    n = len({k.split("_")[1] for k in golden.files if k.startswith("proj_")})
    for i in range(n):
        T, K = (int(v) for v in golden[f"proj_{i}_TK"])
        yield T, K, golden[f"proj_{i}_in"], golden[f"proj_{i}_out"]


def test_project_f64_bit_exact_golden(gpulib, torch_cuda, golden):
    torch = torch_cuda
    for T, K, xin, xref in _proj_cases(golden):
        x = _dev(torch, xin, torch.float64)
        assert gpulib.pasc_gb300_project_f64(C.c_void_p(x.data_ptr()), T, K, None) == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(x.cpu().numpy(), xref, err_msg=f"K={K}")


@pytest.mark.parametrize("K", [1, 2, 3, 4, 5, 7, 8, 13, 32, 100])
def test_project_f64_bit_exact_random(gpulib, torch_cuda, oracle, K):
    torch = torch_cuda
    rng = np.random.default_rng(100 + K)
    T = 20011
    xin = rng.normal(size=T * K) * rng.choice([1e-3, 1.0, 50.0], size=T * K)
    x = _dev(torch, xin, torch.float64)
    assert gpulib.pasc_gb300_project_f64(C.c_void_p(x.data_ptr()), T, K, None) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(x.cpu().numpy(), oracle.project(xin, T, K))


@pytest.mark.parametrize("K", [1, 2, 3, 4, 5, 6, 7, 8, 9, 12, 16, 17, 24, 32])
def test_project_f32_vs_oracle(gpulib, torch_cuda, oracle, K):
    torch = torch_cuda
    rng = np.random.default_rng(200 + K)
    T = 30001
    xin = (rng.normal(size=T * K) * 0.7).astype(np.float32)
    x = _dev(torch, xin, torch.float32)
    assert gpulib.pasc_gb300_project_f32(C.c_void_p(x.data_ptr()), T, K, None) == 0
    torch.cuda.synchronize()
    ref = oracle.project(xin.astype(np.float64), T, K)
    got = x.cpu().numpy().astype(np.float64)
    assert np.max(np.abs(got - ref)) <= 2e-6
    sums = got.reshape(T, K).sum(axis=1)
    assert np.all(got >= 0.0) and np.max(np.abs(sums - 1.0)) <= 2e-6


def test_project_f32_feasible_blocks_untouched(gpulib, torch_cuda):
    torch = torch_cuda
    T, K = 1000, 4
    xin = np.tile(np.array([0.5, 0.25, 0.125, 0.125], dtype=np.float32), T)
    x = _dev(torch, xin, torch.float32)
    assert gpulib.pasc_gb300_project_f32(C.c_void_p(x.data_ptr()), T, K, None) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(x.cpu().numpy(), xin)


def test_project_rejects_bad_k(gpulib):
    assert gpulib.pasc_gb300_project_f32(None, 10, 33, None) != 0
    assert gpulib.pasc_gb300_project_f64(None, 10, 129, None) != 0
    assert gpulib.pasc_gb300_project_f64(None, 0, 3, None) == 0  # empty input is a no-op


@pytest.mark.parametrize("T,K", [(1, 1), (1, 3), (2, 2), (3, 1), (17, 4), (100003, 3)])
def test_matmult_f64_bit_exact(gpulib, torch_cuda, oracle, T, K):
    torch = torch_cuda
    rng = np.random.default_rng(T * 7 + K)
    xin = rng.normal(size=T * K)
    x = _dev(torch, xin, torch.float64)
    y = torch.empty_like(x)
    assert gpulib.pasc_gb300_fem_h1_matmult_f64(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                                T, K, 0.37, None) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(y.cpu().numpy(), oracle.matmult(xin, T, K, 0.37))


def test_matmult_golden(gpulib, torch_cuda, golden):
    torch = torch_cuda
    n = len({k.split("_")[1] for k in golden.files if k.startswith("matmult_")})
    for i in range(n):
        T, K, c = golden[f"matmult_{i}_TKc"]
        x = _dev(torch, golden[f"matmult_{i}_in"], torch.float64)
        y = torch.empty_like(x)
        assert gpulib.pasc_gb300_fem_h1_matmult_f64(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                                    int(T), int(K), float(c), None) == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(y.cpu().numpy(), golden[f"matmult_{i}_out"])


@pytest.mark.parametrize("T,K", [(1, 2), (5, 3), (300001, 3), (4096, 8)])
def test_matmult_f32(gpulib, torch_cuda, oracle, T, K):
    torch = torch_cuda
    rng = np.random.default_rng(T + K)
    xin = rng.normal(size=T * K).astype(np.float32)
    x = _dev(torch, xin, torch.float32)
    y = torch.empty_like(x)
    assert gpulib.pasc_gb300_fem_h1_matmult_f32(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                                T, K, C.c_float(0.37), None) == 0
    torch.cuda.synchronize()
    ref = oracle.matmult(xin.astype(np.float64), T, K, 0.37)
    got = y.cpu().numpy().astype(np.float64)
    scale = max(1e-30, np.max(np.abs(ref)))
    assert np.max(np.abs(got - ref)) <= 1e-6 * scale
