"""The oracle's graph (R > 1) and image mode on the CPU.  The reference implements the graph
operator only as a PETSc matrix assembly (blockgraphsparse.cpp:7-103) and the graphs as
BGMGraph classes; the pins are literal Python transcriptions of those loops on one rank: the
grid and threshold neighbour lists, the assembled matrix (MatSetValue loop, columns summed in
PETSc's sorted order from 0, bit for bit), Decomposition::permute_TRK, and the limits (no
edges: the 1-D operator; R = 1: the 1-D solver).  The solves are checked by their KKT
conditions and, on a two-region image, by the recovered regions."""
import numpy as np
import pytest

from pasc_inference_gb300 import datagen


def _grid2d_transcribed(width, height):
    # bgmgraphgrid2D.h:88-142: left, right, down, up
    nb = []
    for idx in range(width * height):
        i = int(idx / width)
        j = idx - i * width
        lst = []
        if j > 0:
            lst.append(idx - 1)
        if j < width - 1:
            lst.append(idx + 1)
        if i > 0:
            lst.append(idx - width)
        if i < height - 1:
            lst.append(idx + width)
        nb.append(lst)
    return nb


def _threshold_transcribed(coords, n, dim, thr):
    # bgmgraph.cpp:73-152
    nb = [[] for _ in range(n)]
    for i in range(n):
        for j in range(i + 1, n):
            s = 0.0
            for d in range(dim):
                s += (coords[i + d * n] - coords[j + d * n]) * (coords[i + d * n] - coords[j + d * n])
            if s < thr * thr:
                nb[i].append(j)
                nb[j].append(i)
    return nb


def _csr_lists(ptr, idx):
    return [list(idx[ptr[r]:ptr[r + 1]]) for r in range(len(ptr) - 1)]


def _assembled_rows(T, R, K, nb):
    """blockgraphsparse.cpp:48-103: {row: {col: value}} with INSERT_VALUES semantics."""
    rows = {}
    coeff = 1.0
    for k in range(K):
        for r in range(R):
            for t in range(T):
                diag = t * R * K + r * K + k
                m = len(nb[r])
                if t == 0 or t == T - 1:
                    Wsum = 2 * m + 2 if T > 1 else m
                else:
                    Wsum = 3 * m + 4 if T > 1 else m + 1
                row = rows.setdefault(diag, {})
                row[diag] = coeff * Wsum
                if T > 1:
                    if t > 0:
                        row[diag - R * K] = -2 * coeff
                    if t < T - 1:
                        row[diag + R * K] = -2 * coeff
                for rn in nb[r]:
                    idx2 = t * R * K + rn * K + k
                    row[idx2] = -coeff
                    if t > 0:
                        row[idx2 - R * K] = -coeff
                    if t < T - 1:
                        row[idx2 + R * K] = -coeff
    return rows


def _matmult_transcribed(x, T, R, K, nb, coeff):
    rows = _assembled_rows(T, R, K, nb)
    y = np.empty(T * R * K)
    for i in range(T * R * K):
        s = 0.0
        for c in sorted(rows[i]):  # PETSc AIJ rows hold sorted columns
            s += rows[i][c] * x[c]
        y[i] = coeff * s
    return y


@pytest.mark.parametrize("w,h", [(1, 1), (1, 5), (4, 1), (3, 2), (7, 5)])
def test_grid2d_lists(oracle, w, h):
    ptr, idx = oracle.graph_grid2d(w, h)
    ref = _grid2d_transcribed(w, h)
    got = _csr_lists(ptr, idx)
    assert [sorted(l) for l in ref] == got
    assert ptr[-1] == 2 * (h * (w - 1) + w * (h - 1))


def test_grid1d_lists(oracle):
    ptr, idx = oracle.graph_grid1d(6)
    assert _csr_lists(ptr, idx) == [[1], [0, 2], [1, 3], [2, 4], [3, 5], [4]]


@pytest.mark.parametrize("n,dim,thr", [(1, 2, 1.0), (30, 2, 0.3), (50, 3, 0.5), (40, 1, 0.05)])
def test_threshold_lists(oracle, n, dim, thr):
    rng = np.random.default_rng(n * dim)
    c = rng.random(n * dim)
    ptr, idx = oracle.graph_threshold(c, n, dim, thr)
    assert _csr_lists(ptr, idx) == _threshold_transcribed(c, n, dim, thr)


@pytest.mark.parametrize("T,w,h,K", [(1, 4, 3, 2), (1, 1, 1, 3), (2, 3, 3, 2), (5, 4, 2, 3), (6, 1, 1, 2)])
def test_graph_matmult_transcription(oracle, T, w, h, K):
    ptr, idx = oracle.graph_grid2d(w, h)
    R = w * h
    x = np.random.default_rng(T * 100 + R).standard_normal(T * R * K)
    y = oracle.graph_matmult(x, T, K, 0.7, ptr, idx)
    assert np.array_equal(y, _matmult_transcribed(x, T, R, K, _csr_lists(ptr, idx), 0.7))


def test_graph_matmult_threshold_graph(oracle):
    rng = np.random.default_rng(3)
    n, T, K = 25, 4, 3
    c = rng.random(2 * n)
    ptr, idx = oracle.graph_threshold(c, n, 2, 0.35)
    x = rng.standard_normal(T * n * K)
    y = oracle.graph_matmult(x, T, K, 1.3, ptr, idx)
    assert np.array_equal(y, _matmult_transcribed(x, T, n, K, _csr_lists(ptr, idx), 1.3))


def test_graph_limits(oracle):
    T, K = 50, 3
    x = np.random.default_rng(1).standard_normal(T * K)
    ptr = np.zeros(2, dtype=np.int32)
    idx = np.zeros(0, dtype=np.int32)
    # one node, no edges: the 1-D operator, bit for bit
    assert np.array_equal(oracle.graph_matmult(x, T, K, 0.3, ptr, idx), oracle.matmult(x, T, K, 0.3))
    # R nodes without edges: R independent chains
    R = 4
    ptr = np.zeros(R + 1, dtype=np.int32)
    xr = np.random.default_rng(2).standard_normal(T * R * K)
    y = oracle.graph_matmult(xr, T, K, 0.3, ptr, idx).reshape(T, R, K)
    for r in range(R):
        xc = xr.reshape(T, R, K)[:, r, :].ravel()
        assert np.array_equal(y[:, r, :].ravel(), oracle.matmult(xc, T, K, 0.3))


def test_graph_operator_symmetric_psd(oracle):
    T, w, h, K = 3, 4, 3, 2
    ptr, idx = oracle.graph_grid2d(w, h)
    n = T * w * h * K
    A = np.stack([oracle.graph_matmult(np.eye(n)[i], T, K, 1.0, ptr, idx) for i in range(n)], axis=1)
    assert np.array_equal(A, A.T)
    assert np.linalg.eigvalsh(A).min() > -1e-12
    assert np.allclose(A @ np.ones(n), 0.0)  # rows sum to zero


def test_permute_TRK(oracle):
    T, R, K = 5, 3, 2
    v = np.arange(T * R * K, dtype=float)
    out = oracle.permute_TRK(v, T, R, K)
    # decomposition.cpp:260-340 on one rank: new[t*R*K + i*K + k] = orig[k*R*T + i*T + t]
    ref = np.empty_like(v)
    for k in range(K):
        for i in range(R):
            for t in range(T):
                ref[t * R * K + i * K + k] = v[k * R * T + i * T + t]
    assert np.array_equal(out, ref)
    assert np.array_equal(oracle.permute_TRK(v, T * R, 1, K), oracle.permute_blocked_to_interleaved(v, T * R, K))


def _kkt(x, g, nb, K):
    G = g.reshape(nb, K)
    X = x.reshape(nb, K)
    worst = 0.0
    for s in range(nb):
        sup = X[s] > 1e-9
        mu = G[s][sup].min()
        worst = max(worst, float(np.max(np.abs(G[s][sup] - mu))), float(max(0.0, mu - G[s].min())))
    return worst


def test_spgqp_graph_kkt(oracle):
    T, w, h, K = 3, 8, 6, 3
    ptr, idx = oracle.graph_grid2d(w, h)
    nb = T * w * h
    rng = np.random.default_rng(4)
    b = -rng.random(nb * K)
    x0 = oracle.project(rng.random(nb * K), nb, K)
    x, r = oracle.spgqp_solve_graph(b, x0, T, K, 0.05, ptr, idx, oracle.spg_opts(maxit=20000, eps=1e-15))
    g = oracle.graph_matmult(x, T, K, 0.05, ptr, idx) - b
    assert _kkt(x, g, nb, K) < 1e-6
    assert r.fx == pytest.approx(0.5 * x @ (g - b), rel=1e-12)


def _two_region_image(w, h, seed=0, sigma=0.4):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    truth = (((xx - w / 2) ** 2 + (yy - h / 2) ** 2) < (min(w, h) / 3) ** 2).astype(np.int32).ravel()
    data = truth.astype(float) + sigma * rng.standard_normal(w * h)
    return data, truth


def test_image_tssolver_recovers_regions(oracle):
    w, h, K = 40, 30, 2
    data, truth = _two_region_image(w, h)
    ptr, idx = oracle.graph_grid2d(w, h)
    R = w * h
    g0 = datagen.uniform(7, 0, R * K)
    g, th, r = oracle.tssolver_solve_graph(data, g0, np.zeros(K), 1, K, 2.0, ptr, idx,
                                           ts=oracle.ts_opts(maxit=100, eps=1e-10),
                                           spg=oracle.spg_opts(maxit=5000, eps=1e-12))
    lab = np.argmax(g.reshape(R, K), axis=1)
    acc = max(np.mean(lab == truth), np.mean(lab == 1 - truth))
    assert acc > 0.99
    # without the graph coupling (epssqr = 0) the noisy pixels are misclassified more often
    g0b, thb, rb = oracle.tssolver_solve_graph(data, g0, np.zeros(K), 1, K, 0.0, ptr, idx,
                                               ts=oracle.ts_opts(maxit=100, eps=1e-10),
                                               spg=oracle.spg_opts(maxit=5000, eps=1e-12))
    labb = np.argmax(g0b.reshape(R, K), axis=1)
    accb = max(np.mean(labb == truth), np.mean(labb == 1 - truth))
    assert acc > accb


def test_spgqp_coeff_variant(oracle):
    """SPGQPSolverC: with the coefficient factored out the iteration differs from SPGQPSolver
    only in the first step (alphainit / coeff instead of alphainit), the sigma1 clamp and the
    unscaled d'Ad of the stopping tests; both reach the same minimiser."""
    T, K = 800, 3
    sig = datagen.signal1d(T, K, [0.0, 1.0, 2.0], 50, 200, 0.5, 9)
    theta = np.array([0.0, 1.0, 2.0])
    b = oracle.residual_b(sig.data, theta, T, K)
    x0 = datagen.normalised_gamma(sig.gamma0, T, K)
    coeff = oracle.A_coeff(30.0, T)
    o = oracle.spg_opts(maxit=20000, eps=1e-14, m=10)
    xa, ra, _ = oracle.spgqp_solve(b, x0, T, K, coeff, o)
    xc, rc = oracle.spgqp_solve_coeff(b, x0, T, K, coeff, o)
    assert rc.fx == pytest.approx(ra.fx, rel=1e-9)
    assert np.max(np.abs(xa - xc)) < 1e-4
    # coeff = 1: the two loops are the same loop (the first step is alphainit in both)
    xa1, ra1, _ = oracle.spgqp_solve(b, x0, T, K, 1.0, oracle.spg_opts(maxit=50, eps=0.0, m=10))
    xc1, rc1 = oracle.spgqp_solve_coeff(b, x0, T, K, 1.0, oracle.spg_opts(maxit=50, eps=0.0, m=10))
    assert np.array_equal(xa1, xc1) and ra1.fx == rc1.fx
    # on a graph
    ptr, idx = oracle.graph_grid2d(20, 15)
    R = 300
    bg = -np.random.default_rng(2).random(R * K)
    x0g = oracle.project(np.random.default_rng(3).random(R * K), R, K)
    xg, rg = oracle.spgqp_solve_graph(bg, x0g, 1, K, 0.7, ptr, idx, oracle.spg_opts(maxit=20000, eps=1e-14, m=10))
    xgc, rgc = oracle.spgqp_solve_coeff(bg, x0g, 1, K, 0.7, oracle.spg_opts(maxit=20000, eps=1e-14, m=10), ptr, idx)
    assert rgc.fx == pytest.approx(rg.fx, rel=1e-9)
