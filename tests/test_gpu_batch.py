"""Batched solver: many independent signals (own T, K, epssqr) advanced by one launch per SPG
iteration, checked signal by signal against the FP64 oracle.

Tolerances are those of the single-signal mixed path (the batch runs the same per-tile
arithmetic; only the order of its block sums differs): converged objectives within 1e-6
relative of FP64, fixed-length trajectories within 2e-6, TSSolver fixed points with L within
1e-6, theta within 1e-5 of its scale and labels equal on >= 99.99% of timesteps."""
import numpy as np
import pytest

from pasc_inference_gb300 import Batch, capi, datagen

pytestmark = pytest.mark.gpu

# sizes around the tile (504 owned timesteps) and segment (4032 timesteps) boundaries, T = 1
# (A = 0) and every supported K
SPG_CASES = [(1, 3, 5.0), (2, 2, 5.0), (3, 3, 10.0), (503, 2, 10.0), (504, 3, 100.0), (505, 4, 20.0),
             (4031, 3, 30.0), (4032, 2, 10.0), (4033, 5, 50.0), (9000, 3, 1000.0), (2500, 8, 5.0),
             (700, 1, 10.0), (1500, 6, 15.0), (1200, 7, 3.0)]


def _qp(T, K, eps2, seed, oracle):
    rng = np.random.default_rng(seed)
    data = rng.normal(size=T) * 0.5 + rng.integers(0, K, size=T)
    theta = np.arange(K, dtype=float)
    x0 = rng.random(T * K)
    b = oracle.residual_b(data, theta, T, K)
    return data, theta, x0, b, oracle.A_coeff(eps2, T)


def _load(cases, oracle, seed0=0):
    T = [c[0] for c in cases]
    K = [c[1] for c in cases]
    E = [c[2] for c in cases]
    bt = Batch(T, K, E)
    probs = []
    for i, (t, k, e) in enumerate(cases):
        data, theta, x0, b, coeff = _qp(t, k, e, 1000 * seed0 + 17 * i + t, oracle)
        bt.set_data(i, data)
        bt.set_theta(i, theta)
        bt.set_gamma(i, x0)
        probs.append((data, theta, x0, b, coeff))
    return bt, probs


def _fx(oracle, g, b, T, K, coeff):
    return 0.5 * g @ oracle.matmult(g, T, K, coeff) - b @ g


def test_batch_converged_objective(gpulib, oracle):
    bt, probs = _load(SPG_CASES, oracle)
    with bt:
        st = bt.spgqp_solve(capi.spgqp_opts(maxit=3000, stop_difff=0))
        for i, (T, K, _) in enumerate(SPG_CASES):
            data, theta, x0, b, coeff = probs[i]
            if T == 1:
                # A = 0: a linear program over one simplex whose optimum is a single residual,
                # -min_k (x - theta_k)^2; the solver holds x in FP32 and that rounding alone
                # moves one residual by ~1e-6 relative, so the optimum is taken for the stored x
                b32 = oracle.residual_b(data.astype(np.float32).astype(np.float64), theta, T, K)
                f_ref = -np.max(b32)
            else:
                b32 = b
                f_ref = oracle.spgqp_solve(b, x0, T, K, coeff, oracle.spg_opts(maxit=5000, eps=1e-13))[1].fx
            s = st[i]
            assert s.status != capi.PASC_SPG_NONFINITE, (T, K)
            assert abs(s.fx - f_ref) <= 1e-6 * max(abs(f_ref), 1e-12), (T, K, s.fx, f_ref, s.it, s.status)
            g = bt.get_gamma(i)
            G = g.reshape(T, K)
            assert np.all(G >= 0.0) and np.max(np.abs(G.sum(axis=1) - 1.0)) <= 1e-5, (T, K)
            # the reported objective is the objective of the returned gamma: a signal whose solve
            # ended was not touched by the sweeps that followed
            assert abs(_fx(oracle, g, b32, T, K, coeff) - s.fx) <= 1e-6 * max(abs(f_ref), 1e-12), (T, K)


def test_batch_first_iterations_track_oracle(gpulib, oracle):
    cases = [(4000, 3, 20.0), (1000, 2, 5.0), (6000, 5, 100.0), (333, 8, 50.0)]
    for maxit in (0, 1, 3, 10):
        bt, probs = _load(cases, oracle, seed0=maxit)
        with bt:
            st = bt.spgqp_solve(capi.spgqp_opts(maxit=maxit))
            for i, (T, K, _) in enumerate(cases):
                data, theta, x0, b, coeff = probs[i]
                _, ro, _ = oracle.spgqp_solve(b, x0.astype(np.float32).astype(np.float64), T, K, coeff,
                                              oracle.spg_opts(maxit=maxit))
                assert st[i].it == maxit and st[i].status == capi.PASC_SPG_MAXIT
                assert abs(st[i].fx - ro.fx) <= 2e-6 * abs(ro.fx), (maxit, T, K, st[i].fx, ro.fx)


def test_batch_signals_stop_independently(gpulib, oracle):
    """With the reference's default stop rule every signal ends at its own iteration; each
    keeps hessmult == it + 1 and an objective equal to that of its returned gamma."""
    cases = [(3000, 3, 30.0), (500, 2, 2.0), (8000, 4, 300.0), (1200, 3, 10.0), (20000, 2, 50.0)]
    bt, probs = _load(cases, oracle, seed0=7)
    with bt:
        st = bt.spgqp_solve(capi.spgqp_opts(eps=1e-6, m=10, maxit=20000))
        its = [s.it for s in st]
        assert len(set(its)) > 1, its
        for i, (T, K, _) in enumerate(cases):
            data, theta, x0, b, coeff = probs[i]
            assert st[i].status == capi.PASC_SPG_CONVERGED, (i, st[i].status)
            assert st[i].hessmult == st[i].it + 1
            g = bt.get_gamma(i)
            assert abs(_fx(oracle, g, b, T, K, coeff) - st[i].fx) <= 1e-6 * abs(st[i].fx), i


TS_CASES = [(dict(T=4000, K=3, levels=[0.0, 1.0, 2.0], smin=200, smax=800, sigma=0.5, seed=3), 20.0),
            (dict(T=3000, K=2, levels=[1.0, 2.0], smin=200, smax=600, sigma=0.8, seed=21), 10.0),
            (dict(T=5000, K=3, levels=[0.0, 1.0, 2.0], smin=400, smax=1500, sigma=0.4, seed=11), 300.0),
            (dict(T=5000, K=4, levels=[0.0, 1.0, 2.0, 3.0], smin=100, smax=500, sigma=0.3, seed=12), 5.0),
            (dict(T=900, K=2, levels=[0.0, 3.0], smin=50, smax=200, sigma=0.6, seed=5), 8.0),
            (dict(T=6000, K=5, levels=[0.0, 1.0, 2.0, 3.0, 4.0], smin=300, smax=900, sigma=0.25, seed=9), 30.0)]


def test_batch_tssolver_tight_vs_oracle(gpulib, oracle):
    """Every signal's TSSolver driven to its fixed point (SPG |f - f_old| < 1e-13, outer
    |L - L_old| < 1e-13), all signals in one batch, against the oracle run per signal."""
    sigs = [datagen.signal1d(g["T"], g["K"], g["levels"], g["smin"], g["smax"], g["sigma"], g["seed"])
            for g, _ in TS_CASES]
    eps = [e for _, e in TS_CASES]
    bt = Batch([s.T for s in sigs], [s.K for s in sigs], eps)
    with bt:
        for i, s in enumerate(sigs):
            bt.set_data(i, s.data)
            bt.set_gamma(i, s.gamma0)
            bt.set_theta(i, np.zeros(s.K))
        st = bt.ts_solve(capi.ts_opts(maxit=300, eps=1e-13), capi.spgqp_opts(m=10, eps=1e-13, maxit=20000))
        for i, s in enumerate(sigs):
            T, K = s.T, s.K
            g_o, th_o, r_o, _ = oracle.tssolver_solve(s.data, s.gamma0, np.zeros(K), T, K, eps[i],
                                                      ts=oracle.ts_opts(maxit=300, eps=1e-13),
                                                      spg=oracle.spg_opts(m=10, eps=1e-13, maxit=20000))
            th = bt.get_theta(i)
            g = bt.get_gamma(i)
            assert abs(st[i].L - r_o.L) <= 1e-6 * abs(r_o.L), (i, st[i].L, r_o.L)
            assert np.max(np.abs(th - th_o)) <= 1e-5 * np.max(np.abs(th_o)), (i, th, th_o)
            lab = np.argmax(g.reshape(T, K), axis=1)
            lab_o = np.argmax(g_o.reshape(T, K), axis=1)
            assert np.mean(lab == lab_o) >= 0.9999, i


def test_batch_uneven_256_consistency(gpulib, oracle):
    """The 256-signal workload of uneven signals (T log-uniform in [1e3, 1e6], K in 2..5,
    epssqr log-uniform in [1, 1000]) with the reference's default settings: every signal's
    outer loop ends, gamma is feasible, and each reported L is the objective of the returned
    gamma under the returned theta, evaluated in FP64 on the host."""
    inst = datagen.batched()
    bt = Batch([s.T for s in inst], [s.K for s in inst], [s.epssqr for s in inst])
    with bt:
        for i, s in enumerate(inst):
            bt.set_data(i, s.data)
            bt.set_gamma(i, s.gamma0)
            bt.set_theta(i, np.zeros(s.K))
        st = bt.ts_solve(capi.ts_opts(), capi.spgqp_opts(m=10, eps=1e-6))
        rng = np.random.default_rng(0)
        for i in sorted(rng.choice(len(inst), size=48, replace=False)):
            s = inst[i]
            T, K = s.T, s.K
            assert st[i].it_last < 300 and np.isfinite(st[i].L), (i, st[i].it_last)
            g = bt.get_gamma(i)
            th = bt.get_theta(i)
            G = g.reshape(T, K)
            assert np.all(G >= 0.0) and np.max(np.abs(G.sum(axis=1) - 1.0)) <= 1e-5, i
            b = oracle.residual_b(s.data, th, T, K)
            L_host = _fx(oracle, g, b, T, K, oracle.A_coeff(s.epssqr, T))
            assert abs(L_host - st[i].L) <= 1e-6 * abs(st[i].L), (i, L_host, st[i].L)


def test_batch_bad_arguments(gpulib):
    with pytest.raises(capi.PascError):
        Batch([100, 200], [3, 9], [1.0, 1.0])
    with pytest.raises(capi.PascError):
        Batch([0], [3], [1.0])
    with pytest.raises(ValueError):
        Batch([100, 200], [3], [1.0, 1.0])
    with Batch([100, 200], [3, 2], [1.0, 1.0]) as bt:
        with pytest.raises(capi.PascError):
            bt.set_data(2, np.zeros(100))
        with pytest.raises(capi.PascError):
            bt.set_theta(-1, np.zeros(3))
        with pytest.raises(capi.PascError):
            bt.spgqp_solve(capi.spgqp_opts(stop_normgp_normb=1))
        with pytest.raises(capi.PascError):
            bt.ts_solve(capi.ts_opts(annealing=3))


def _ts_batch(sigs, epssqr, device_loop, chunk=4, theta0=None, **ts_kw):
    bt = Batch([s.T for s in sigs], [s.K for s in sigs], epssqr)
    bt.set_loop(device_loop, chunk)
    for i, s in enumerate(sigs):
        bt.set_data(i, s.data)
        bt.set_gamma(i, s.gamma0)
        bt.set_theta(i, np.zeros(s.K) if theta0 is None else theta0[i])
    st = bt.ts_solve(capi.ts_opts(**ts_kw), capi.spgqp_opts(m=10, eps=1e-9, maxit=5000))
    out = [(x.L, x.it_last, x.spg_it_sum, x.L_increased, bt.get_theta(i), bt.get_gamma(i)) for i, x in enumerate(st)]
    bt.close()
    return out


@pytest.mark.parametrize("chunk", [1, 4, 7])
def test_batch_device_loop_equals_host_loop(gpulib, chunk):
    """The device-driven loops (one graph launch per solve, conditional WHILE nodes, control
    on the device every `chunk` sweeps) make exactly the iterations of the host-driven loop:
    every signal's SPG and TSSolver results are bit-identical (each signal's sweeps do not
    depend on how the sweeps are grouped)."""
    sigs = [datagen.signal1d(g["T"], g["K"], g["levels"], g["smin"], g["smax"], g["sigma"], g["seed"])
            for g, _ in TS_CASES]
    eps = [e for _, e in TS_CASES]
    host = _ts_batch(sigs, eps, False, maxit=50, eps=1e-9)
    dev = _ts_batch(sigs, eps, True, chunk, maxit=50, eps=1e-9)
    for i, (h, d) in enumerate(zip(host, dev)):
        assert h[:4] == d[:4], (i, h[:4], d[:4])
        np.testing.assert_array_equal(h[4], d[4])
        np.testing.assert_array_equal(h[5], d[5])
    # theta given (TSSolver::set_solution_theta): the graph without the theta step
    th = [np.linspace(0.0, 2.0, s.K) for s in sigs]
    host = _ts_batch(sigs, eps, False, theta0=th, maxit=3, thetasolved=1)
    dev = _ts_batch(sigs, eps, True, chunk, theta0=th, maxit=3, thetasolved=1)
    for h, d in zip(host, dev):
        assert h[:4] == d[:4]
        np.testing.assert_array_equal(h[5], d[5])


def test_batch_device_loop_spg_equals_host_loop(gpulib, oracle):
    res = []
    for device_loop in (False, True):
        bt, probs = _load(SPG_CASES, oracle, seed0=3)
        with bt:
            bt.set_loop(device_loop, 4)
            st = bt.spgqp_solve(capi.spgqp_opts(m=10, eps=1e-10, maxit=4000))
            res.append(([(s.it, s.status, s.fx) for s in st], [bt.get_gamma(i) for i in range(len(SPG_CASES))]))
            st0 = bt.spgqp_solve(capi.spgqp_opts(maxit=0))  # maxit 0: the set-up only
            assert all(s.it == 0 and s.status == capi.PASC_SPG_MAXIT for s in st0)
    assert res[0][0] == res[1][0]
    for a, b in zip(res[0][1], res[1][1]):
        np.testing.assert_array_equal(a, b)


def test_batch_set_loop_arguments(gpulib):
    with Batch([100, 200], [3, 2], [1.0, 1.0]) as bt:
        with pytest.raises(capi.PascError):
            bt.set_loop(True, 0)
        with pytest.raises(capi.PascError):
            bt.set_loop(True, 65)
        bt.set_loop(False, 1)
        bt.set_loop(True, 64)


def test_batch_work_items_automatic_and_pinned(gpulib, oracle):
    """Work items sized from the segments still running (the default, and with another number
    of items per block) and fixed segment sizes give the same converged objectives (the item
    size changes only the grouping of the block partials in the per-signal sums)."""
    fx = {}
    for tiles in (0, -1, -16, 2, 32):
        bt, probs = _load(SPG_CASES, oracle, seed0=5)
        with bt:
            bt.set_segment_tiles(tiles)
            st = bt.spgqp_solve(capi.spgqp_opts(maxit=3000, stop_difff=0))
            seg, item = bt.get_segment_tiles()
            if tiles <= 0:
                assert seg == 4 and item % 4 == 0 and 4 <= item <= 32, (tiles, seg, item)
            else:
                assert seg == item == tiles
            fx[tiles] = np.array([s.fx for s in st])
    for tiles in (-1, -16, 2, 32):
        np.testing.assert_allclose(fx[tiles], fx[0], rtol=1e-6, atol=1e-12)
    with Batch([100, 200], [3, 2], [1.0, 1.0]) as bt:
        for bad in (1, 65, -17):
            with pytest.raises(capi.PascError):
                bt.set_segment_tiles(bad)


def test_batch_items_merge_with_many_segments(gpulib):
    """With every signal long enough that the list is merged (items of several segments), the
    automatic list and the same solve with one segment per item agree: the per-signal sums
    collect every item exactly once (a lost or doubled item would change f)."""
    sigs = [datagen.signal1d(T, 3, [0.0, 1.0, 2.0], 500, 5000, 0.5, 40 + q)
            for q, T in enumerate([6_000_000, 4_000_000, 2_500_000, 900_000, 3_000])]
    fx = {}
    for tiles in (0, -1, 4):
        with Batch([s.T for s in sigs], [3] * len(sigs), [10.0] * len(sigs)) as bt:
            bt.set_segment_tiles(tiles)
            for i, s in enumerate(sigs):
                bt.set_data(i, s.data)
                bt.set_gamma(i, s.gamma0)
                bt.set_theta(i, np.array([0.0, 1.0, 2.0]))
            st = bt.spgqp_solve(capi.spgqp_opts(maxit=200, stop_difff=0))
            fx[tiles] = np.array([x.fx for x in st])
            if tiles <= 0:
                assert bt.get_segment_tiles()[1] > 4
    np.testing.assert_allclose(fx[0], fx[4], rtol=1e-6)
    np.testing.assert_allclose(fx[-1], fx[4], rtol=1e-6)


def test_batch_retuned_after_solves_keeps_theta(gpulib):
    """Changing the segment size after a TSSolver run (whose theta steps updated the device
    copy of every signal's theta) keeps those thetas: the objective of the final gamma,
    evaluated by a zero-iteration solve, is the same with and without the change."""
    sigs = [datagen.signal1d(g["T"], g["K"], g["levels"], g["smin"], g["smax"], g["sigma"], g["seed"])
            for g, _ in TS_CASES]
    eps = [e for _, e in TS_CASES]
    fx = []
    for relayout in (False, True):
        with Batch([s.T for s in sigs], [s.K for s in sigs], eps) as bt:
            bt.set_segment_tiles(8)
            for i, s in enumerate(sigs):
                bt.set_data(i, s.data)
                bt.set_gamma(i, s.gamma0)
                bt.set_theta(i, np.zeros(s.K))
            bt.ts_solve(capi.ts_opts(maxit=5), capi.spgqp_opts(m=10, eps=1e-9))
            if relayout:
                bt.set_segment_tiles(2)
            st = bt.spgqp_solve(capi.spgqp_opts(maxit=0))
            fx.append(np.array([x.fx for x in st]))
    np.testing.assert_allclose(fx[1], fx[0], rtol=1e-9)
