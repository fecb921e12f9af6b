"""Host side of the graph (R > 1) / image mode, no GPU needed: the library's graph builders
against the oracle's restatement of BGMGraph / BGMGraphGrid1D / BGMGraphGrid2D, the graph
checks of pasc_gb300_create_graph (rejected before any device work), and the Python mirror's
layout helpers (Decomposition::permute_TRK / permute_TRxdim) against the oracle."""
import ctypes as C

import numpy as np
import pytest

from pasc_inference_gb300 import BGMGraph, BGMGraphGrid1D, BGMGraphGrid2D, Decomposition, capi


@pytest.fixture(scope="module")
def lib():
    from pasc_inference_gb300 import build as B
    B.build()
    return capi.load()


@pytest.mark.parametrize("w,h", [(1, 1), (1, 7), (9, 1), (5, 4), (33, 17)])
def test_grid2d_equals_oracle(lib, oracle, w, h):
    g = BGMGraphGrid2D(w, h)
    g.process_grid()
    ptr, idx = oracle.graph_grid2d(w, h)
    assert np.array_equal(g.ptr, ptr) and np.array_equal(g.idx, idx)
    assert g.get_m() == h * (w - 1) + w * (h - 1)
    assert g.get_m_max() == (0 if w * h == 1 else min(4, int(np.max(np.diff(ptr)))))


@pytest.mark.parametrize("w", [1, 2, 10])
def test_grid1d_equals_oracle(lib, oracle, w):
    g = BGMGraphGrid1D(w)
    g.process_grid()
    ptr, idx = oracle.graph_grid1d(w)
    assert np.array_equal(g.ptr, ptr) and np.array_equal(g.idx, idx)


@pytest.mark.parametrize("n,dim,thr", [(1, 2, 1.0), (60, 2, 0.25), (80, 3, 0.4), (50, 1, 0.02)])
def test_threshold_equals_oracle(lib, oracle, n, dim, thr):
    c = np.random.default_rng(n + dim).random(n * dim)
    g = BGMGraph(c, n, dim)
    g.process(thr)
    ptr, idx = oracle.graph_threshold(c, n, dim, thr)
    assert np.array_equal(g.ptr, ptr) and np.array_equal(g.idx, idx)


def test_threshold_size_query_and_capacity(lib):
    c = np.random.default_rng(0).random(40)
    ptr = np.empty(21, dtype=np.int32)
    nnz = C.c_long()
    assert lib.pasc_gb300_graph_threshold(c, 20, 2, 0.5, ptr, None, 0, C.byref(nnz)) == 0
    assert nnz.value == ptr[-1] > 0
    small = np.empty(1, dtype=np.int32)
    assert lib.pasc_gb300_graph_threshold(c, 20, 2, 0.5, ptr, small.ctypes.data, 1, C.byref(nnz)) == capi.PASC_ERR_ARG
    assert lib.pasc_gb300_graph_grid2d(0, 3, ptr, small) == capi.PASC_ERR_ARG


BAD_GRAPHS = [
    ("self loop", [0, 1, 2], [0, 0]),
    ("unsorted", [0, 2, 3, 4], [2, 1, 0, 0]),
    ("duplicate", [0, 2, 4], [1, 1, 0, 0]),
    ("out of range", [0, 1, 2], [5, 0]),
    ("asymmetric", [0, 1, 1], [1]),
    ("bad offsets", [1, 1, 2], [0, 0]),
    ("decreasing", [0, 2, 1], [1, 0]),
]


@pytest.mark.parametrize("name,ptr,idx", BAD_GRAPHS, ids=[b[0] for b in BAD_GRAPHS])
def test_create_graph_rejects_bad_graphs(lib, name, ptr, idx):
    h = C.c_void_p()
    ptr = np.array(ptr, dtype=np.int32)
    idx = np.array(idx, dtype=np.int32)
    rc = lib.pasc_gb300_create_graph(C.byref(h), 10, len(ptr) - 1, 2, 0, 1.0, 0, ptr, idx)
    assert rc == capi.PASC_ERR_ARG, name
    assert b"create_graph" in lib.pasc_gb300_last_error()
    assert not h.value


def test_create_graph_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    g = BGMGraphGrid2D(3, 3)
    g.process_grid()
    h = C.c_void_p()
    rc = lib.pasc_gb300_create_graph(C.byref(h), 1, 9, 2, 0, 1.0, 0, g.ptr, g.idx)
    assert rc == capi.PASC_ERR_CUDA and not h.value


def test_decomposition_layouts(oracle):
    T, R, K = 4, 6, 3
    g = BGMGraphGrid2D(3, 2)
    g.process_grid()
    dec = Decomposition(T, g, K)
    assert dec.get_R() == 6 and dec.get_graph() is g
    v = np.arange(T * R * K, dtype=float)
    assert np.array_equal(dec.permute_TRK(v), oracle.permute_TRK(v, T, R, K))
    assert np.array_equal(dec.permute_TRK(dec.permute_TRK(v), invert=True), v)
    d = np.arange(T * R, dtype=float)
    assert np.array_equal(dec.permute_TRxdim(d).reshape(T, R), d.reshape(R, T).T)
    # R > 1 without a graph: disjoint nodes (graphh1fem.cpp:30-45)
    dec2 = Decomposition(T, 5, K)
    assert dec2.get_graph().get_m() == 0 and dec2.get_graph().get_n() == 5


def test_imagedata_layout_and_data_ops(tmp_path):
    """ImageData reads node-major pixels (r*T + t) into the interleaved layout t*R + r; the
    TSData preprocessing (cutdata, scaledata / unscaledata, shiftdata; tsdata.cpp:384-560) on
    the host copy, before a model exists."""
    from pasc_inference_gb300 import ImageData, petscio
    T, w, h, K = 3, 4, 2, 2
    g = BGMGraphGrid2D(w, h)
    g.process_grid()
    dec = Decomposition(T, g, K)
    raw = np.arange(T * w * h, dtype=float)
    path = str(tmp_path / "img.bin")
    petscio.save_vec(path, raw)
    img = ImageData(dec, path, w, h)
    assert np.array_equal(img.get_datavector().reshape(T, w * h), raw.reshape(w * h, T).T)
    with pytest.raises(capi.PascError):
        ImageData(dec, raw[:-1], w, h)
    img.cutdata(2.0, 20.0)
    d = img.get_datavector()
    assert d.min() == 2.0 and d.max() == 20.0
    img.scaledata(-1.0, 1.0)
    d = img.get_datavector()
    assert d.min() == pytest.approx(-1.0) and d.max() == pytest.approx(1.0)
    img.unscaledata(-1.0, 1.0)
    assert np.allclose(img.get_datavector().reshape(T, w * h), np.clip(raw, 2, 20).reshape(w * h, T).T)
    img.shiftdata(0.5)
    assert img.get_datavector().min() == pytest.approx(2.5)
