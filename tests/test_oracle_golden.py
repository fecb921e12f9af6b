"""The FP64 oracle against golden vectors produced by the reference's own code
(tests/golden/make_golden.py runs the reference's SPGQPSolver / TSSolver / SPG_fs /
SimplexFeasibleSet_Local compiled from its sources).  Bit-exact: the oracle restates the
reference's operation order."""
import numpy as np
import pytest


def _n(golden, prefix):
    return len({k.split("_")[1] for k in golden.files if k.startswith(prefix + "_")})


def test_projection_matches_reference(oracle, golden):
    for i in range(_n(golden, "proj")):
        T, K = (int(v) for v in golden[f"proj_{i}_TK"])
        got = oracle.project(golden[f"proj_{i}_in"], T, K)
        np.testing.assert_array_equal(got, golden[f"proj_{i}_out"], err_msg=f"case {i} K={K}")


def test_matmult_matches_reference(oracle, golden):
    for i in range(_n(golden, "matmult")):
        T, K, c = golden[f"matmult_{i}_TKc"]
        got = oracle.matmult(golden[f"matmult_{i}_in"], int(T), int(K), c)
        np.testing.assert_array_equal(got, golden[f"matmult_{i}_out"])


def _fs_python(m, vals):
    # src/general/solver/spg_fs.cpp:17-63 restated
    fs = [vals[0]] * m
    last = 0
    out = [max(fs)]
    for v in vals[1:]:
        last += 1
        if last >= m:
            last = 0
        fs[last] = v
        out.append(max(fs))
    return np.array(out)


def test_gll_memory_matches_reference(golden):
    for i in range(_n(golden, "fs")):
        m = int(golden[f"fs_{i}_m"][0])
        np.testing.assert_array_equal(_fs_python(m, golden[f"fs_{i}_in"]), golden[f"fs_{i}_out"])


_OPTMAP = {"spgqpsolver_m": "m", "spgqpsolver_eps": "eps", "spgqpsolver_maxit": "maxit",
           "spgqpsolver_stop_difff": "stop_difff", "spgqpsolver_stop_normgp": "stop_normgp",
           "spgqpsolver_gamma": "gamma", "spgqpsolver_alphainit": "alphainit",
           "spgqpsolver_sigma2": "sigma2"}


def test_spgqp_matches_reference(oracle, golden):
    for i in range(_n(golden, "spg")):
        T, K, coeff = golden[f"spg_{i}_TKc"]
        T, K = int(T), int(K)
        kw = {}
        for name, val in zip(golden[f"spg_{i}_optnames"], golden[f"spg_{i}_optvals"]):
            if name:
                f = _OPTMAP[str(name)]
                kw[f] = int(val) if f in ("m", "maxit", "stop_difff", "stop_normgp") else float(val)
        x, r, _ = oracle.spgqp_solve(golden[f"spg_{i}_b"], golden[f"spg_{i}_x0"], T, K, coeff,
                                     oracle.spg_opts(**kw))
        it, hm, fx = golden[f"spg_{i}_res"]
        assert r.it == int(it) and r.hessmult == int(hm), f"case {i}"
        assert r.fx == fx, f"case {i}: {r.fx!r} != {fx!r}"
        np.testing.assert_array_equal(x, golden[f"spg_{i}_x"])


def test_tssolver_matches_reference(oracle, golden):
    for i in range(_n(golden, "ts")):
        T, K, eps2 = golden[f"ts_{i}_TKe"]
        T, K = int(T), int(K)
        g, th, r, _ = oracle.tssolver_solve(golden[f"ts_{i}_data"], golden[f"ts_{i}_gamma0"],
                                            np.zeros(K), T, K, eps2)
        L, it_last, it_sum, aic = golden[f"ts_{i}_res"]
        name = str(golden[f"ts_{i}_name"][0])
        assert r.L == L, name
        assert r.it_last == int(it_last) and r.it_sum == int(it_sum), name
        assert r.aic == aic, name
        np.testing.assert_array_equal(th, golden[f"ts_{i}_theta"], err_msg=name)
        np.testing.assert_array_equal(g, golden[f"ts_{i}_gamma"], err_msg=name)
