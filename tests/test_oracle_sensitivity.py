"""Sensitivity of the reference's alternating loop to rounding, measured on the FP64 oracle
alone: the batched workload's signals (T log-uniform in [1e3, 1e6], K in 2..5, epssqr
log-uniform in [1, 1000]) solved from their random gamma0 and from gamma0 perturbed by 1e-7
relative (the size of one FP32 rounding), with the batch line's stopping rules (SPG
|f - f_old| < 1e-6, m 10; outer loop to 1e-6 relative change of L).  The first theta step from a
random gamma makes the K levels nearly equal, and perturbations at rounding level decide where
the loop ends, so L moves far more than 1e-6 on most signals.  The batched mixed solver's L
against the plain FP64 path is therefore compared as a distribution, not signal by signal.

    python tests/test_oracle_sensitivity.py [n]   # the summary on the n smallest signals"""
import sys

import numpy as np


def relative_L_changes(O, n):
    from pasc_inference_gb300 import datagen
    order = np.argsort(datagen.batched_lengths(), kind="stable")[:n]
    inst = datagen.batched(indices=order)
    ts = O.ts_opts(eps=1e-6, relative=1)
    spg = O.spg_opts(m=10, eps=1e-6)
    rel = []
    for i, s in zip(order, inst):
        _, _, r1, _ = O.tssolver_solve(s.data, s.gamma0, np.zeros(s.K), s.T, s.K, s.epssqr, ts=ts, spg=spg)
        u = datagen.uniform(99, int(i), s.gamma0.size)
        g1 = s.gamma0 * (1.0 + 1e-7 * (2.0 * u - 1.0))
        _, _, r2, _ = O.tssolver_solve(s.data, g1, np.zeros(s.K), s.T, s.K, s.epssqr, ts=ts, spg=spg)
        rel.append(abs(r2.L - r1.L) / abs(r1.L))
    return np.array(rel)


def test_rounding_level_perturbation_moves_L(oracle):
    rel = relative_L_changes(oracle, 12)
    assert np.mean(rel <= 1e-6) <= 0.5, rel
    assert np.max(rel) >= 1e-4, rel


if __name__ == "__main__":
    import os
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import pasc_oracle as O
    O.build()
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 48
    r = relative_L_changes(O, n)
    print(f"signals {n}: median {np.median(r):.2e}, max {np.max(r):.2e}, "
          f"within 1e-6 {np.mean(r <= 1e-6):.0%}, within 1e-4 {np.mean(r <= 1e-4):.0%}")
