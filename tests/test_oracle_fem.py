"""The oracle's FEM temporal coarsening (Fem / FemHat reduce and prolongate, the reduced gamma
step of GraphH1FEMModel) on the CPU.  The reference's FEM code exists only as PETSc
specialisations that cannot be built here, so the pins are: a hand-computed FEM-SUM case, the
partition and sum properties of FEM-SUM, a second, literal Python transcription of the
reference's FEM-HAT loops (femhat.cpp:64-100, 150-171, femhat.h:154-195 on one rank), and the
unreduced limit (fem_reduce = 1) equal to the plain TSSolver."""
import math

import numpy as np
import pytest

from pasc_inference_gb300 import datagen


def test_fem_sum_hand_case(oracle):
    # T1 = 5, T2 = 2: diff = 2.5, blocks [round(0), round(2.5)) = [0, 3) and [3, 5)
    g1 = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    assert np.array_equal(oracle.fem_reduce(g1, 5, 2, 1, 0), [6.0, 9.0])
    assert np.array_equal(oracle.fem_prolongate(np.array([7.0, 8.0]), 5, 2, 1, 0), [7, 7, 7, 8, 8])


@pytest.mark.parametrize("T1", [7, 100, 1001, 4096])
@pytest.mark.parametrize("r", [0.1, 0.33, 0.5, 0.9, 0.999])
def test_fem_sum_partition(oracle, T1, r):
    K = 3
    T2 = oracle.fem_T_reduced(T1, r)
    assert T2 == math.ceil(T1 * r)
    g = np.random.default_rng(T1).random(T1 * K)
    g2 = oracle.fem_reduce(g, T1, T2, K, 0)
    assert np.allclose(g2.reshape(T2, K).sum(axis=0), g.reshape(T1, K).sum(axis=0), rtol=1e-12)
    # prolongation of the reduction of a block-constant field is that field
    c = oracle.fem_prolongate(np.arange(T2 * K, dtype=float), T1, T2, K, 0)
    blocks = oracle.fem_reduce(np.ones(T1 * K), T1, T2, K, 0)  # block lengths
    assert np.array_equal(oracle.fem_reduce(c, T1, T2, K, 0), np.arange(T2 * K) * blocks)


def _hat_reduce_transcribed(g1, T1, T2, K):
    diff = (T1 - 1) / (T2 - 1)
    right_t1_idx = math.floor(diff * (T2 - 1))
    g2 = np.zeros(T2 * K)
    for k in range(K):
        for t2 in range(T2):
            center, left, right = t2 * diff, (t2 - 1) * diff, (t2 + 1) * diff
            id_counter = math.floor(left)
            t1 = math.floor(left)
            mysum = 0.0
            while t1 <= center:
                phi = (t1 - left) / (center - left)
                if id_counter >= 0:
                    mysum += phi * g1[id_counter * K + k]
                t1 += 1
                id_counter += 1
            while t1 < right:
                phi = (t1 - right) / (center - right)
                if id_counter < right_t1_idx:
                    mysum += phi * g1[id_counter * K + k]
                t1 += 1
                id_counter += 1
            g2[t2 * K + k] = mysum
    return g2


def _hat_prolongate_transcribed(g2, T1, T2, K):
    diff = (T1 - 1) / (T2 - 1)
    g1 = np.zeros(T1 * K)
    for k in range(K):
        for t1 in range(T1):
            l = math.floor(t1 / diff)
            r = l + 1
            tl, tr = l * diff, r * diff
            pl = (t1 - tl) / (tr - tl)
            pr = (t1 - tr) / (tl - tr)
            v = 0.0
            v += pl * (g2[r * K + k] if r < T2 else 0.0)
            v += pr * (g2[l * K + k] if l < T2 else 0.0)
            g1[t1 * K + k] = v
    return g1


@pytest.mark.parametrize("T1,r", [(11, 0.5), (100, 0.3), (257, 0.9), (64, 0.25), (1000, 0.07)])
def test_fem_hat_matches_transcription(oracle, T1, r):
    K = 2
    T2 = oracle.fem_T_reduced(T1, r)
    g = np.random.default_rng(T1 + 1).random(T1 * K)
    assert np.array_equal(oracle.fem_reduce(g, T1, T2, K, 1), _hat_reduce_transcribed(g, T1, T2, K))
    g2 = np.random.default_rng(T1 + 2).random(T2 * K)
    assert np.array_equal(oracle.fem_prolongate(g2, T1, T2, K, 1), _hat_prolongate_transcribed(g2, T1, T2, K))
    # linear interpolation reproduces constants
    assert np.allclose(oracle.fem_prolongate(np.ones(T2 * K), T1, T2, K, 1), 1.0)


def test_unreduced_limit_equals_tssolver(oracle):
    sig = datagen.signal1d(3000, 3, [0.0, 1.0, 2.0], 200, 600, 0.5, 3)
    ts = oracle.ts_opts(maxit=50, eps=1e-9)
    spg = oracle.spg_opts(m=10, eps=1e-9)
    g_a, th_a, r_a, _ = oracle.tssolver_solve(sig.data, sig.gamma0, np.zeros(3), 3000, 3, 20.0, ts=ts, spg=spg)
    g_b, th_b, r_b = oracle.tssolver_solve_fem(sig.data, sig.gamma0, np.zeros(3), 3000, 3, 20.0, 1.0, 0, ts=ts, spg=spg)
    assert r_a.L == r_b.L and np.array_equal(th_a, th_b) and np.array_equal(g_a, g_b)


@pytest.mark.parametrize("fem_type", [0, 1])
def test_reduced_tssolver_runs(oracle, fem_type):
    sig = datagen.signal1d(4000, 3, [0.0, 1.0, 2.0], 200, 800, 0.5, 4)
    g, th, r = oracle.tssolver_solve_fem(sig.data, sig.gamma0, np.zeros(3), 4000, 3, 20.0, 0.25, fem_type,
                                         ts=oracle.ts_opts(maxit=100), spg=oracle.spg_opts(m=10))
    assert np.isfinite(r.L) and r.it_last < 100
    G = g.reshape(4000, 3)
    assert np.all(np.isfinite(G))
    if fem_type == 0:  # block copies of simplex points are simplex points
        assert np.all(G >= 0) and np.allclose(G.sum(axis=1), 1.0)
    assert np.max(np.abs(np.sort(th) - [0.0, 1.0, 2.0])) < 0.1
