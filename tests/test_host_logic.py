"""Host-side logic without a GPU: seeded generators, PETSc binary I/O, the option mapping of
the reference-style classes, and the replica timing helpers over two gloo ranks."""
import os
import socket
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from pasc_inference_gb300 import datagen, petscio, spg_opts_from, ts_opts_from, Decomposition, PascError

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_generator_is_deterministic_and_shaped():
    a = datagen.uniform(5, 1, 1000)
    b = datagen.uniform(5, 1, 1000)
    np.testing.assert_array_equal(a, b)
    assert a.min() >= 0.0 and a.max() < 1.0
    assert abs(a.mean() - 0.5) < 0.05
    # counter-based: a window equals the slice of the full stream
    np.testing.assert_array_equal(datagen.uniform(5, 1, 10, offset=500), a[500:510])
    z = datagen.normal(9, 2, 200_000)
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01


def test_signal_configs():
    s0 = datagen.signal1d_cfg0()
    assert s0.T == 10_000 and s0.K == 2 and s0.gamma0.size == 20_000
    lens = np.diff(np.flatnonzero(np.diff(s0.labels)))
    assert lens.min() >= 500 and lens.max() <= 2000
    assert set(np.unique(s0.clean)) <= {1.0, 2.0}
    s1 = datagen.signal1d_cfg1(T=200_000)
    assert s1.K == 3 and set(np.unique(s1.clean)) <= {0.0, 1.0, 2.0}
    assert abs(np.std(s1.data - s1.clean) - 0.5) < 0.01
    b = datagen.batched(8)
    assert all(1000 <= x.T <= 1_000_000 and 2 <= x.K <= 5 and 1 <= x.epssqr <= 1000 for x in b)
    assert all(np.all(np.diff(x.levels) >= 0) for x in b)


def test_normalised_gamma():
    g0 = datagen.uniform(1, 0, 30)
    g = datagen.normalised_gamma(g0, 10, 3).reshape(10, 3)
    np.testing.assert_allclose(g.sum(axis=1), 1.0)


def test_petsc_vec_roundtrip(tmp_path):
    v = np.random.default_rng(0).normal(size=123)
    p = str(tmp_path / "v.bin")
    petscio.save_vec(p, v)
    raw = open(p, "rb").read()
    assert raw[:4] == (1211214).to_bytes(4, "big") and raw[4:8] == (123).to_bytes(4, "big")
    np.testing.assert_array_equal(petscio.load_vec(p), v)


def test_reference_option_names():
    o = spg_opts_from({"spgqpsolver_m": 10, "spgqpsolver_eps": 1e-6, "spgqpsolver_stop_normgp": True})
    assert (o.m, o.eps, o.stop_normgp) == (10, 1e-6, 1)
    t = ts_opts_from({"tssolver_maxit": 5, "tssolver_init_permute": False})
    assert (t.maxit, t.init_permute) == (5, 0)


def test_decomposition_limits():
    d = Decomposition(100, 1, 3, 1, 1)
    assert (d.get_T(), d.get_K(), d.get_R()) == (100, 3, 1)
    # R > 1 nodes without a graph: disjoint nodes (graph mode); multichannel graph data refused
    d4 = Decomposition(100, 4, 3, 1, 1)
    assert d4.get_R() == 4 and d4.get_graph().get_m() == 0
    with pytest.raises(PascError):
        Decomposition(100, 4, 3, 2, 1)
    with pytest.raises(PascError):
        Decomposition(100, 1, 3, 1, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_replica_timing_two_gloo_ranks(tmp_path):
    """Two ranks: barrier, max and sum over ranks, as bench.py combines replica timings."""
    pytest.importorskip("torch")
    script = tmp_path / "w.py"
    script.write_text(textwrap.dedent(f"""
        import os, sys, json
        sys.path.insert(0, {ROOT!r})
        import bench
        info = bench.dist_init(timeout_s=60)
        bench.dist_barrier(info)
        mx = bench.max_over_ranks(info, 10.0 + info.rank)
        sm = bench.sum_over_ranks(info, 1.0)
        print(json.dumps({{"rank": info.rank, "ws": info.world_size, "max": mx, "sum": sm}}))
        bench.dist_finalize(info)
    """))
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    import json
    res = [json.loads(o.strip().splitlines()[-1]) for o, _ in outs]
    assert all(r["ws"] == 2 and r["max"] == 11.0 and r["sum"] == 2.0 for r in res)


def test_model_getters_wiring(monkeypatch):
    """GraphH1FEMModel's reference getters (get_T, get_T_reduced, get_fem_reduce, get_L,
    get_linear_quadratic, get_graph, get_epssqr) over a stand-in for the GPU problem."""
    import pasc_inference_gb300 as P

    class FakeProblem:
        def __init__(self, T, K, epssqr, precision=None, xdim=1, device=0, graph=None):
            self.T, self.K, self.R = T, K, 1
            self.calls = []

        def __getattr__(self, name):
            return lambda *a, **k: self.calls.append(name)

        def get_fem(self):
            return 0.25, 0, 250

        def get_fx(self):
            return -1.5

    monkeypatch.setattr(P, "Problem", FakeProblem)
    data = P.Signal1DData(np.linspace(0.0, 1.0, 1000))
    data.set_decomposition(P.Decomposition(1000, 1, 3, 1, 1))
    m = P.GraphH1FEMModel(data, 7.0, fem=P.Fem(0.25))
    assert (m.get_T(), m.get_T_reduced(), m.get_fem_reduce(), m.get_epssqr()) == (1000, 250, 0.25, 7.0)
    assert m.get_L() == -1.5 and m.get_linear_quadratic() == (0.0, 0.0)
    assert m.get_graph() is None  # a 1-D signal has no graph
    assert "set_fem" in m.problem.calls
    m2 = P.GraphH1FEMModel(data, 7.0)
    assert m2.get_T_reduced() == 1000 and m2.get_fem_reduce() == 1.0


def test_vector_sizes_are_checked_before_the_abi():
    """The Python mirror refuses arrays shorter than what the ABI will read (PASC_ERR_ARG),
    and hands through the caller's array without a copy when it fits (page-locked buffers
    stay page-locked)."""
    import pasc_inference_gb300 as P
    from pasc_inference_gb300 import capi
    p = object.__new__(P.Problem)
    p._h, p.T, p.K, p.xdim = None, 10, 3, 1
    for call, n in ((p.set_data, 10), (p.set_gamma, 30), (p.set_theta, 3), (p.recon_mse, 10),
                    (p.abserr_reconstructed, 10)):
        with pytest.raises(capi.PascError) as e:
            call(np.zeros(n - 1))
        assert e.value.code == capi.PASC_ERR_ARG and "values expected" in str(e.value)
        with pytest.raises(capi.PascError) as e:  # right size: reaches the ABI, which refuses the NULL handle
            call(np.zeros(n))
        assert "values expected" not in str(e.value)
    x = np.arange(30.0)
    assert np.shares_memory(P._vec(x, 30, "x"), x)
    b = object.__new__(P.Batch)
    b._h, b.n, b.T, b.K = None, 2, np.array([5, 7]), np.array([2, 3], dtype=np.int32)
    with pytest.raises(capi.PascError) as e:
        b.set_gamma(1, np.zeros(20))
    assert "values expected" in str(e.value)
    with pytest.raises(capi.PascError) as e:
        b.set_gamma(1, np.zeros(21))
    assert "values expected" not in str(e.value)
    with pytest.raises(capi.PascError) as e:  # an index outside the batch is the ABI's to refuse
        b.set_theta(-1, np.zeros(3))
    assert "values expected" not in str(e.value)
