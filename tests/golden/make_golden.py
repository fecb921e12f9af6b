"""Generates tests/golden/golden_ref.npz from the reference's own code.

Run with the PASC_inference tree named on the command line (or in $PASC_REFERENCE):
  python tests/golden/make_golden.py <PASC_inference tree>
It builds oracle/_ref/libpasc_ref.so (oracle/build_ref.sh: the reference's generic
SPGQPSolver / TSSolver / SPG_fs / SimplexFeasibleSet_Local templates compiled unmodified
against host-array shims) and records inputs and outputs of:
  proj_*     SimplexFeasibleSet_Local::project on random and hand-made blocks
  matmult_*  the FEM-H1 operator as the shim assembles it (pins the row-sum order)
  fs_*       SPG_fs init/update/get_max sequences
  spg_*      SPGQPSolver::solve on small QPs (default and non-default settings)
  ts_*       TSSolver::solve with the FEM-H1 model hooks on
             - the reference's test vectors Matlab/signal1D_scalability/tests/small_data.bin
               and small_gamma0.bin (T=1000, K=2; gamma0 used as the set_random values),
             - the first 2000 samples of examples/test_signal1D/data/samplesignal.bin,
             - the synthetic T = 1e4, K = 2 signal (levels {1, 2}) of pasc_inference_gb300.datagen.
The fixtures let the CPU tests pin the oracle to the reference without the reference tree.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import pasc_oracle as O  # noqa: E402
from pasc_inference_gb300 import datagen  # noqa: E402
from pasc_inference_gb300.petscio import load_vec  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PASC_REFERENCE", "")
if not os.path.isfile(os.path.join(REF, "include/general/solver/spgqpsolver.h")):
    sys.exit("make_golden: give the PASC_inference tree as the first argument or in PASC_REFERENCE")
os.environ["PASC_REFERENCE"] = REF  # oracle/build_ref.sh compiles from the same tree
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_ref.npz")


def proj_cases(rng):
    cases = []
    for K in (1, 2, 3, 4, 5, 8, 13, 32):
        T = 64
        x = rng.normal(size=T * K) * 1.5
        x[: 2 * K] = np.abs(x[: 2 * K])
        # already feasible rows
        for t in (3, 5):
            v = rng.random(K)
            x[t * K:(t + 1) * K] = v / v.sum()
        # ties, one dominant, all equal, exactly-sum-1 with a negative entry
        x[7 * K:8 * K] = 0.25
        x[9 * K:10 * K] = 0.0
        x[9 * K] = 5.0
        if K >= 2:
            x[11 * K:12 * K] = 0.5
            x[11 * K] = -0.5
            x[11 * K + 1] = 1.5 - 0.5 * (K - 2)
        cases.append((K, T, x))
    return cases


def main():
    if not os.path.exists(os.path.join(REF, "include/general/solver/spgqpsolver.h")):
        sys.exit(f"reference tree not found at {REF}")
    O.build()
    if O.build_ref() is None:
        sys.exit("oracle/_ref could not be built")
    rng = np.random.default_rng(20241203)
    out = {}

    for i, (K, T, x) in enumerate(proj_cases(rng)):
        out[f"proj_{i}_in"] = x
        out[f"proj_{i}_TK"] = np.array([T, K])
        out[f"proj_{i}_out"] = O.ref_project(x, T, K)

    for i, (T, K) in enumerate([(1, 1), (1, 3), (2, 2), (3, 1), (5, 3), (17, 4)]):
        x = rng.normal(size=T * K)
        out[f"matmult_{i}_in"] = x
        out[f"matmult_{i}_TKc"] = np.array([T, K, 0.37])
        out[f"matmult_{i}_out"] = O.ref_matmult(x, T, K, 0.37)

    for i, m in enumerate((1, 3, 10, 20)):
        vals = rng.normal(size=60)
        out[f"fs_{i}_m"] = np.array([m])
        out[f"fs_{i}_in"] = vals
        out[f"fs_{i}_out"] = O.ref_fs_sequence(m, vals)

    spg_cases = [
        dict(T=300, K=2, eps2=10.0, opts={}),
        dict(T=500, K=3, eps2=100.0, opts={"spgqpsolver_m": 10, "spgqpsolver_eps": 1e-6}),
        dict(T=200, K=4, eps2=1.0, opts={"spgqpsolver_maxit": 25}),
        dict(T=1, K=4, eps2=5.0, opts={}),
        dict(T=2, K=2, eps2=5.0, opts={}),
        dict(T=400, K=3, eps2=50.0, opts={"spgqpsolver_stop_difff": 0, "spgqpsolver_stop_normgp": 1,
                                          "spgqpsolver_eps": 1e-10}),
        dict(T=300, K=5, eps2=20.0, opts={"spgqpsolver_gamma": 0.5, "spgqpsolver_alphainit": 0.5,
                                          "spgqpsolver_sigma2": 0.8}),
    ]
    for i, c in enumerate(spg_cases):
        T, K = c["T"], c["K"]
        data = rng.normal(size=T) + rng.integers(0, K, size=T)
        theta = np.arange(K, dtype=float)
        b = O.residual_b(data, theta, T, K)
        x0 = rng.random(T * K)
        coeff = O.A_coeff(c["eps2"], T)
        x, it, hm, fx = O.ref_spgqp_solve(b, x0, T, K, coeff, **c["opts"])
        out[f"spg_{i}_b"] = b
        out[f"spg_{i}_data"] = data
        out[f"spg_{i}_theta"] = theta
        out[f"spg_{i}_x0"] = x0
        out[f"spg_{i}_TKc"] = np.array([T, K, coeff])
        out[f"spg_{i}_optnames"] = np.array(list(c["opts"].keys()) or [""])
        out[f"spg_{i}_optvals"] = np.array(list(c["opts"].values()) or [0.0], dtype=float)
        out[f"spg_{i}_x"] = x
        out[f"spg_{i}_res"] = np.array([it, hm, fx])

    ts_cases = []
    d = load_vec(os.path.join(REF, "Matlab/signal1D_scalability/tests/small_data.bin"))
    g0 = load_vec(os.path.join(REF, "Matlab/signal1D_scalability/tests/small_gamma0.bin"))
    ts_cases.append(("small_data_eps10", d, g0, 2, 10.0))
    ts_cases.append(("small_data_eps1000", d, g0, 2, 1000.0))
    s = load_vec(os.path.join(REF, "examples/test_signal1D/data/samplesignal.bin"))[:2000]
    ts_cases.append(("samplesignal2000_eps10", s, rng.random(2 * 2000), 2, 10.0))
    sig = datagen.signal1d_cfg0()
    ts_cases.append(("cfg0_eps10", sig.data, sig.gamma0, 2, 10.0))
    s3 = datagen.signal1d(3000, 3, [0.0, 1.0, 2.0], 100, 600, 0.5, seed=7)
    ts_cases.append(("k3_eps50", s3.data, s3.gamma0, 3, 50.0))
    for i, (name, data, gam, K, eps2) in enumerate(ts_cases):
        T = data.size
        g, th, res = O.ref_tssolver_solve(data, gam, np.zeros(K), T, K, eps2)
        out[f"ts_{i}_name"] = np.array([name])
        out[f"ts_{i}_data"] = data
        out[f"ts_{i}_gamma0"] = gam
        out[f"ts_{i}_TKe"] = np.array([T, K, eps2])
        out[f"ts_{i}_gamma"] = g
        out[f"ts_{i}_theta"] = th
        out[f"ts_{i}_res"] = np.array([res["L"], res["it_last"], res["it_sum"], res["aic"]])
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1024:.0f} KiB)")


if __name__ == "__main__":
    main()
