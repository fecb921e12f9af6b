"""GB300-native FEM-H1 time-series clustering: the host-side mirror of the reference's
class surface over the C ABI of include/pasc_gb300.h.

Class names, constructor arguments and option names follow PASC_inference:
  Decomposition(T, R | graph, K, xdim, DD_size)  include/general/common/decomposition.h:55
  BGMGraph, BGMGraphGrid1D, BGMGraphGrid2D       include/general/algebra/graph/
  ImageData(decomposition, filename, width, height)   include/general/data/imagedata.h
  Signal1DData(filename | array)                 include/general/data/signal1Ddata.h
  GraphH1FEMModel(tsdata, epssqr, fem=None, usethetainpenalty=False)
                                                 include/general/model/graphh1fem.h:75
  TSSolver(tsdata, annealing=1)                  include/general/solver/tssolver.h:80-104
  SPGQPSolver (reached as TSSolver.get_gammasolver())   include/general/solver/spgqpsolver.h:118-151
Options use the reference's console keys (spgqpsolver_maxit, tssolver_eps, ...), passed as a
dict.  All computation runs on the GPU through libpasc_gb300.so; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import (PASC_PREC_FP64, PASC_PREC_MIXED, PascError, SpgqpOpts, SpgqpStats, TsOpts,
                   TsStats, check, load)

__all__ = ["Problem", "Batch", "Fem", "FemHat", "Decomposition", "Signal1DData", "TSData", "GraphH1FEMModel", "TSSolver",
           "SPGQPSolver", "BGMGraph", "BGMGraphGrid1D", "BGMGraphGrid2D", "ImageData", "PascError",
           "PASC_PREC_FP64", "PASC_PREC_MIXED", "capi"]

_SPG_KEYS = {"spgqpsolver_maxit": "maxit", "spgqpsolver_eps": "eps", "spgqpsolver_m": "m",
             "spgqpsolver_gamma": "gamma", "spgqpsolver_sigma1": "sigma1",
             "spgqpsolver_sigma2": "sigma2", "spgqpsolver_alphainit": "alphainit",
             "spgqpsolver_stop_difff": "stop_difff", "spgqpsolver_stop_normgp": "stop_normgp",
             "spgqpsolver_stop_normgp_normb": "stop_normgp_normb",
             "spgqpsolver_stop_Anormgp": "stop_Anormgp",
             "spgqpsolver_stop_Anormgp_normb": "stop_Anormgp_normb"}
_TS_KEYS = {"tssolver_maxit": "maxit", "tssolver_eps": "eps",
            "tssolver_init_permute": "init_permute"}


def spg_opts_from(options: dict | None) -> SpgqpOpts:
    o = capi.spgqp_opts()
    for k, v in (options or {}).items():
        if k in _SPG_KEYS:
            setattr(o, _SPG_KEYS[k], type(getattr(o, _SPG_KEYS[k]))(v))
    return o


def ts_opts_from(options: dict | None) -> TsOpts:
    o = capi.ts_opts()
    for k, v in (options or {}).items():
        if k in _TS_KEYS:
            setattr(o, _TS_KEYS[k], type(getattr(o, _TS_KEYS[k]))(v))
    return o


def _vec(a, n: int, what: str) -> np.ndarray:
    """a as a contiguous float64 array of exactly n values: the ABI reads n values from the
    pointer it gets, so an array of another size is refused here (PASC_ERR_ARG), as the C++
    mirror refuses it; pass a slice where a prefix is meant."""
    v = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    if v.size != n:
        raise PascError(capi.PASC_ERR_ARG, f"{what}: {n} values expected, got {v.size}")
    return v


def _vec32(a, n: int, what: str) -> np.ndarray:
    """a as a contiguous float32 array of exactly n values (PASC_ERR_ARG otherwise)."""
    v = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    if v.size != n:
        raise PascError(capi.PASC_ERR_ARG, f"{what}: {n} values expected, got {v.size}")
    return v


class Problem:
    """One FEM-H1 problem on one GPU (a pasc_gb300_problem handle)."""

    def __init__(self, T: int, K: int, epssqr: float = 1.0, precision: int = PASC_PREC_MIXED,
                 xdim: int = 1, device: int = 0, graph=None):
        """graph: (nbr_ptr, nbr_idx) CSR neighbour lists of R nodes (or a BGMGraph) for the
        graph / image mode; T then counts timesteps and the problem has T*R blocks of K."""
        L = load()
        h = C.c_void_p()
        self.Ttime, self.R = int(T), 1
        if graph is not None:
            ptr, idx = graph.csr() if hasattr(graph, "csr") else graph
            ptr = np.ascontiguousarray(ptr, dtype=np.int32)
            idx = np.ascontiguousarray(idx, dtype=np.int32)
            if idx.size == 0:
                idx = np.zeros(1, dtype=np.int32)
            if xdim != 1:
                raise PascError(capi.PASC_ERR_NOTSUPP, "graph problems take scalar data (xdim 1)")
            self.R = len(ptr) - 1
            check(L.pasc_gb300_create_graph(C.byref(h), int(T), self.R, int(K), int(precision), float(epssqr),
                                            int(device), ptr, idx))
        else:
            check(L.pasc_gb300_create(C.byref(h), int(T), int(K), int(xdim), int(precision),
                                      float(epssqr), int(device)))
        self._h = h
        # T counts the blocks of K (timesteps x nodes), as the handle does
        self.T, self.K, self.xdim, self.precision = int(T) * self.R, int(K), int(xdim), int(precision)
        self.epssqr = float(epssqr)

    def close(self):
        if getattr(self, "_h", None):
            load().pasc_gb300_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # TSData vectors
    def set_epssqr(self, epssqr: float, scalef: bool = True):
        self.epssqr = float(epssqr)
        check(load().pasc_gb300_set_epssqr(self._h, float(epssqr), 1 if scalef else 0))

    def set_data(self, data):
        check(load().pasc_gb300_set_data(self._h, _vec(data, self.T * self.xdim, "set_data")))

    def set_gamma(self, gamma):
        check(load().pasc_gb300_set_gamma(self._h, _vec(gamma, self.T * self.K, "set_gamma")))

    def get_gamma(self) -> np.ndarray:
        out = np.empty(self.T * self.K)
        check(load().pasc_gb300_get_gamma(self._h, out))
        return out

    def get_gamma_into(self, out: np.ndarray) -> np.ndarray:
        """get_gamma into a caller's array (e.g. page-locked host memory)."""
        if out.dtype != np.float64 or out.size != self.T * self.K or not out.flags.c_contiguous:
            raise ValueError("get_gamma_into: a contiguous float64 array of T*K values is needed")
        check(load().pasc_gb300_get_gamma(self._h, out))
        return out

    def set_data_f32(self, data):
        """set_data from FP32 values (the mixed path's device format: half the bytes, no
        conversion)."""
        check(load().pasc_gb300_set_data_f32(self._h, _vec32(data, self.T * self.xdim, "set_data_f32")))

    def set_gamma_f32(self, gamma):
        check(load().pasc_gb300_set_gamma_f32(self._h, _vec32(gamma, self.T * self.K, "set_gamma_f32")))

    def get_gamma_f32_into(self, out: np.ndarray) -> np.ndarray:
        """gamma as FP32 values into a caller's array (e.g. page-locked host memory)."""
        if out.dtype != np.float32 or out.size != self.T * self.K or not out.flags.c_contiguous:
            raise ValueError("get_gamma_f32_into: a contiguous float32 array of T*K values is needed")
        check(load().pasc_gb300_get_gamma_f32(self._h, out))
        return out

    def set_theta(self, theta):
        check(load().pasc_gb300_set_theta(self._h, _vec(theta, self.K * self.xdim, "set_theta")))

    def get_theta(self) -> np.ndarray:
        out = np.empty(self.K * self.xdim)
        check(load().pasc_gb300_get_theta(self._h, out))
        return out

    # model hooks
    def permute_gamma(self):
        check(load().pasc_gb300_permute_gamma(self._h))

    def update_theta(self):
        check(load().pasc_gb300_update_theta(self._h))

    def update_b(self):
        check(load().pasc_gb300_update_b(self._h))

    # solvers
    def spgqp_solve(self, opts: SpgqpOpts | None = None) -> SpgqpStats:
        st = SpgqpStats()
        check(load().pasc_gb300_spgqp_solve(self._h, C.byref(opts or capi.spgqp_opts()), C.byref(st)))
        return st

    def spgqp_start(self, opts: SpgqpOpts | None = None):
        check(load().pasc_gb300_spgqp_start(self._h, C.byref(opts or capi.spgqp_opts())))

    def spgqp_iterate(self, n: int, poll: bool = True) -> SpgqpStats:
        st = SpgqpStats()
        check(load().pasc_gb300_spgqp_iterate(self._h, int(n), 1 if poll else 0, C.byref(st)))
        return st

    def spgqp_last_iterate(self):
        ms = C.c_double()
        n = C.c_int()
        check(load().pasc_gb300_spgqp_last_iterate(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def set_sweep_variant(self, variant: int):
        check(load().pasc_gb300_set_sweep_variant(self._h, int(variant)))

    def get_sweep_variant(self) -> int:
        v = C.c_int()
        check(load().pasc_gb300_get_sweep_variant(self._h, C.byref(v)))
        return v.value

    def get_sweep_tuning(self):
        """(kernel, blocks of its grid, tuned sweep time in ms)."""
        v, g, ms = C.c_int(), C.c_int(), C.c_double()
        check(load().pasc_gb300_get_sweep_tuning(self._h, C.byref(v), C.byref(g), C.byref(ms)))
        return v.value, g.value, ms.value

    def time_model_kernels(self, which: int, reps: int = 10) -> float:
        """ms per call of the theta update (which=1) or the residual (which=2)."""
        v = C.c_double()
        check(load().pasc_gb300_time_model_kernels(self._h, int(which), int(reps), C.byref(v)))
        return v.value

    def set_fem(self, fem_reduce: float, fem_type: int = 0):
        """FEM temporal coarsening of the gamma step: 0 FEM-SUM, 1 FEM-HAT; fem_reduce = 1: none."""
        check(load().pasc_gb300_set_fem(self._h, float(fem_reduce), int(fem_type)))

    def get_fem(self):
        """(fem_reduce, fem_type, T of the gamma QP)."""
        r, t, T2 = C.c_double(), C.c_int(), C.c_long()
        check(load().pasc_gb300_get_fem(self._h, C.byref(r), C.byref(t), C.byref(T2)))
        return r.value, t.value, T2.value

    def set_gamma_solver_type(self, t: int):
        """0 automatic (SPGQPSolver), 1 SPGQPSolver, 2 SPGQPSolverC."""
        check(load().pasc_gb300_set_gamma_solver_type(self._h, int(t)))

    def get_gamma_solver_type(self) -> int:
        v = C.c_int()
        check(load().pasc_gb300_get_gamma_solver_type(self._h, C.byref(v)))
        return v.value

    def get_graph(self):
        """(timesteps, nodes, neighbour entries); (T, 1, 0) for a 1-D problem."""
        T, R, nnz = C.c_long(), C.c_long(), C.c_long()
        check(load().pasc_gb300_get_graph(self._h, C.byref(T), C.byref(R), C.byref(nnz)))
        return T.value, R.value, nnz.value

    def set_usethetainpenalty(self, on: bool = True):
        """Theta in the penalty: block k of A scaled by alpha*theta_k^2, theta step with the
        penalty term (xdim 1, no FEM reduction)."""
        check(load().pasc_gb300_set_usethetainpenalty(self._h, 1 if on else 0))

    def get_usethetainpenalty(self) -> bool:
        v = C.c_int()
        check(load().pasc_gb300_get_usethetainpenalty(self._h, C.byref(v)))
        return bool(v.value)

    def get_b(self) -> np.ndarray:
        out = np.empty(self.T * self.K)
        check(load().pasc_gb300_get_b(self._h, out))
        return out

    def set_residual_engine(self, engine: int):
        """Multichannel data: 0 = tensor cores, 1 = CUDA cores."""
        check(load().pasc_gb300_set_residual_engine(self._h, int(engine)))

    def get_residual_engine(self) -> int:
        v = C.c_int()
        check(load().pasc_gb300_get_residual_engine(self._h, C.byref(v)))
        return v.value

    def get_fx(self) -> float:
        v = C.c_double()
        check(load().pasc_gb300_get_fx(self._h, C.byref(v)))
        return v.value

    def ts_solve(self, ts: TsOpts | None = None, spg: SpgqpOpts | None = None,
                 gamma_restart=None) -> TsStats:
        st = TsStats()
        gr = None
        if gamma_restart is not None:
            gr = _vec(gamma_restart, self.T * self.K, "ts_solve gamma_restart")
        check(load().pasc_gb300_ts_solve(self._h, C.byref(ts or capi.ts_opts()),
                                         C.byref(spg or capi.spgqp_opts()),
                                         gr.ctypes.data if gr is not None else None, C.byref(st)))
        return st

    def abserr_reconstructed(self, solution) -> float:
        v = C.c_double()
        check(load().pasc_gb300_abserr_reconstructed(
            self._h, _vec(solution, self.T, "abserr_reconstructed"), C.byref(v)))
        return v.value

    def argmax_labels(self) -> np.ndarray:
        out = np.empty(self.T, dtype=np.int32)
        check(load().pasc_gb300_argmax_labels(self._h, out))
        return out

    # derivatives through the converged gamma step
    def recon_mse(self, clean) -> float:
        v = C.c_double()
        check(load().pasc_gb300_recon_mse(self._h, _vec(clean, self.T, "recon_mse"), C.byref(v)))
        return v.value

    def polish(self, opts: capi.PolishOpts | None = None) -> capi.PolishStats:
        """Refine gamma to the optimum of the QP on the face the solve ended on (FP64
        face-Newton rounds; see pasc_gb300_polish)."""
        st = capi.PolishStats()
        check(load().pasc_gb300_polish(self._h, C.byref(opts or capi.polish_opts()), C.byref(st)))
        return st

    def adjoint(self, dloss_dgamma=None, opts: capi.AdjointOpts | None = None):
        """Returns (dloss/d epssqr, dloss/d data [T], dloss/d theta [K], AdjointStats)."""
        deps = C.c_double()
        ddata = np.empty(self.T)
        dtheta = np.empty(self.K)
        st = capi.AdjointStats()
        g = None if dloss_dgamma is None else _vec(dloss_dgamma, self.T * self.K, "adjoint dloss_dgamma")
        check(load().pasc_gb300_adjoint(self._h, g.ctypes.data if g is not None else None,
                                        C.byref(opts or capi.adjoint_opts()), C.byref(deps),
                                        ddata.ctypes.data, dtheta.ctypes.data, C.byref(st)))
        return deps.value, ddata, dtheta, st


class Batch:
    """n independent signals (own T, K, epssqr) solved together on one GPU (a
    pasc_gb300_batch handle): one launch per SPG iteration for all signals still running."""

    def __init__(self, T, K, epssqr, device: int = 0):
        self.T = np.ascontiguousarray(T, dtype=capi.LONG_DTYPE)
        self.K = np.ascontiguousarray(K, dtype=np.int32)
        eps = np.ascontiguousarray(epssqr, dtype=np.float64)
        if not (len(self.T) == len(self.K) == len(eps)):
            raise ValueError("T, K and epssqr need one entry per signal")
        self.n = len(self.T)
        h = C.c_void_p()
        check(load().pasc_gb300_batch_create(C.byref(h), self.n, self.T, self.K, eps, int(device)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            load().pasc_gb300_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _vec(self, i, a, what: int, name: str):
        """Signal i's array checked against its size (what: 1 data T_i, 2 gamma T_i*K_i, 3 theta
        K_i); an index outside the batch is left to the ABI, which refuses it."""
        i = int(i)
        if not 0 <= i < self.n:
            return np.ascontiguousarray(a, dtype=np.float64)
        T, K = int(self.T[i]), int(self.K[i])
        return _vec(a, {1: T, 2: T * K, 3: K}[what], name)

    def set_loop(self, device_loop: bool = True, chunk: int = 4):
        """device_loop: each solve is one graph launch whose loops are decided on the device
        every `chunk` sweeps (default); False: the host drives the sweeps in chunks."""
        check(load().pasc_gb300_batch_set_loop(self._h, 1 if device_loop else 0, int(chunk)))

    def set_segment_tiles(self, tiles: int = 0):
        """Work items of the batched sweeps: 0 (default) sized at every rebuild of the work list
        from the segments still running (4-tile segments, items of 4 to 32 tiles, about four per
        resident block); -c the same with about c items per resident block; 2..64 fixed items of
        that many tiles."""
        check(load().pasc_gb300_batch_set_segment_tiles(self._h, int(tiles)))

    def get_segment_tiles(self):
        """(tiles per segment, tiles per work item with every signal running)."""
        t, it = C.c_int(), C.c_int()
        check(load().pasc_gb300_batch_get_segment_tiles(self._h, C.byref(t), C.byref(it)))
        return t.value, it.value

    def set_data(self, i: int, data):
        check(load().pasc_gb300_batch_set_data(self._h, int(i), self._vec(i, data, 1, "batch_set_data")))

    def set_gamma(self, i: int, gamma):
        check(load().pasc_gb300_batch_set_gamma(self._h, int(i), self._vec(i, gamma, 2, "batch_set_gamma")))

    def get_gamma(self, i: int) -> np.ndarray:
        out = np.empty(int(self.T[i]) * int(self.K[i]))
        check(load().pasc_gb300_batch_get_gamma(self._h, int(i), out))
        return out

    def set_theta(self, i: int, theta):
        check(load().pasc_gb300_batch_set_theta(self._h, int(i), self._vec(i, theta, 3, "batch_set_theta")))

    def get_theta(self, i: int) -> np.ndarray:
        out = np.empty(int(self.K[i]))
        check(load().pasc_gb300_batch_get_theta(self._h, int(i), out))
        return out

    def spgqp_solve(self, opts: SpgqpOpts | None = None) -> list:
        st = (SpgqpStats * self.n)()
        check(load().pasc_gb300_batch_spgqp_solve(self._h, C.byref(opts or capi.spgqp_opts()), st))
        return list(st)

    def ts_solve(self, ts: TsOpts | None = None, spg: SpgqpOpts | None = None) -> list:
        st = (TsStats * self.n)()
        check(load().pasc_gb300_batch_ts_solve(self._h, C.byref(ts or capi.ts_opts()),
                                               C.byref(spg or capi.spgqp_opts()), st))
        return list(st)


# ------------------------------------------------------------------------------------------
# mirror of the reference classes on the path
# ------------------------------------------------------------------------------------------
class BGMGraph:
    """BGMGraph<VectorBase>: a graph of n nodes given by coordinates (dim values per node,
    stored dimension by dimension, or a PETSc binary file of them), with edges between nodes
    closer than a threshold (process, src/petscvector/algebra/graph/bgmgraph.cpp:73-152).
    Neighbour lists are kept as CSR arrays sorted ascending."""

    def __init__(self, coordinates=None, n: int | None = None, dim: int = 2, filename: str | None = None):
        if filename is not None or isinstance(coordinates, str):
            from .petscio import load_vec
            coordinates = load_vec(filename or coordinates)
        self.coordinates = None if coordinates is None else np.ascontiguousarray(coordinates, dtype=np.float64)
        self.dim = int(dim)
        self.n = int(n) if n is not None else (0 if coordinates is None else self.coordinates.size // self.dim)
        self.threshold = -1.0
        self.processed = False
        self.ptr = None
        self.idx = None

    def process(self, threshold: float):
        L = load()
        ptr = np.empty(self.n + 1, dtype=np.int32)
        nnz = C.c_long()
        check(L.pasc_gb300_graph_threshold(self.coordinates, self.n, self.dim, float(threshold), ptr, None, 0,
                                           C.byref(nnz)))
        idx = np.empty(max(nnz.value, 1), dtype=np.int32)
        check(L.pasc_gb300_graph_threshold(self.coordinates, self.n, self.dim, float(threshold), ptr,
                                           idx.ctypes.data, idx.size, C.byref(nnz)))
        self._set(ptr, idx[: nnz.value], threshold)

    def _set(self, ptr, idx, threshold):
        self.ptr, self.idx = ptr, np.ascontiguousarray(idx, dtype=np.int32)
        self.threshold = float(threshold)
        self.processed = True

    def csr(self):
        if not self.processed:
            raise PascError(capi.PASC_ERR_STATE, "graph not processed")
        return self.ptr, self.idx

    def get_n(self):
        return self.n

    def get_m(self):
        return int(self.ptr[-1]) // 2

    def get_m_max(self):
        return int(np.max(np.diff(self.ptr))) if self.n > 0 else 0

    def get_dim(self):
        return self.dim

    def get_threshold(self):
        return self.threshold

    def get_neighbor_nmbs(self):
        return np.diff(self.ptr)

    def get_neighbor_ids(self):
        return [self.idx[self.ptr[r]:self.ptr[r + 1]] for r in range(self.n)]

    def get_coordinates(self):
        return self.coordinates

    def get_name(self):
        return "BGMGraph"


class BGMGraphGrid1D(BGMGraph):
    """BGMGraphGrid1D<VectorBase>(width): a chain of width nodes (bgmgraphgrid1D.h)."""

    def __init__(self, width: int):
        super().__init__(np.arange(width, dtype=np.float64), width, 1)
        self.width = int(width)

    def process_grid(self):
        ptr = np.empty(self.width + 1, dtype=np.int32)
        idx = np.empty(max(2 * (self.width - 1), 1), dtype=np.int32)
        check(load().pasc_gb300_graph_grid1d(self.width, ptr, idx))
        self._set(ptr, idx[: ptr[-1]], 1.1)

    def get_name(self):
        return "BGMGraphGrid1D"


class BGMGraphGrid2D(BGMGraph):
    """BGMGraphGrid2D<VectorBase>(width, height): the 4-neighbour pixel grid of an image,
    node i*width + j (bgmgraphgrid2D.h:88-142)."""

    def __init__(self, width: int, height: int):
        self.width, self.height = int(width), int(height)
        jj, ii = np.meshgrid(np.arange(width, dtype=np.float64), np.arange(height, dtype=np.float64))
        super().__init__(np.concatenate([jj.ravel(), ii.ravel()]), width * height, 2)

    def process_grid(self):
        n = self.width * self.height
        ptr = np.empty(n + 1, dtype=np.int32)
        idx = np.empty(max(2 * (self.height * (self.width - 1) + self.width * (self.height - 1)), 1), dtype=np.int32)
        check(load().pasc_gb300_graph_grid2d(self.width, self.height, ptr, idx))
        self._set(ptr, idx[: ptr[-1]], 1.1)

    def get_width(self):
        return self.width

    def get_height(self):
        return self.height

    def get_name(self):
        return "BGMGraphGrid2D"


class Decomposition:
    """Decomposition<VectorBase>(T, R, K, xdim, DDT_size) or (T, graph, K, xdim, DDR_size):
    layouts of one GPU.  With R > 1 nodes and no graph the nodes are disjoint (the graph the
    model builds when none is given, graphh1fem.cpp:30-45)."""

    def __init__(self, T: int, R, K: int, xdim: int = 1, DD_size: int = 1):
        if DD_size != 1:
            raise PascError(capi.PASC_ERR_NOTSUPP, "one GPU per problem: DDT_size / DDR_size must be 1")
        if isinstance(R, BGMGraph):
            self.graph = R
            R = R.get_n()
        else:
            self.graph = None
            if int(R) > 1:
                g = BGMGraph(np.arange(int(R), dtype=np.float64), int(R), 1)
                g.process(0.0)
                self.graph = g
        self.T, self.R, self.K, self.xdim = int(T), int(R), int(K), int(xdim)
        if self.R > 1 and self.xdim != 1:
            raise PascError(capi.PASC_ERR_NOTSUPP, "graph problems take scalar data (xdim 1)")

    def get_T(self):
        return self.T

    def get_K(self):
        return self.K

    def get_R(self):
        return self.R

    def get_xdim(self):
        return self.xdim

    def get_graph(self):
        return self.graph

    def permute_TRK(self, v, invert: bool = False):
        """blocked k*R*T + r*T + t <-> interleaved (t*R + r)*K + k (decomposition.cpp:257-340)."""
        T, R, K = self.T, self.R, self.K
        v = np.asarray(v, dtype=np.float64)
        if not invert:
            return v.reshape(K, R, T).transpose(2, 1, 0).ravel().copy()
        return v.reshape(T, R, K).transpose(2, 1, 0).ravel().copy()

    def permute_TRxdim(self, v, invert: bool = False):
        """data: r*T + t (file order) <-> t*R + r."""
        T, R = self.T, self.R
        v = np.asarray(v, dtype=np.float64)
        if not invert:
            return v.reshape(R, T).T.ravel().copy()
        return v.reshape(T, R).T.ravel().copy()


class TSData:
    """TSData<VectorBase>: data, gamma and theta vectors of one time series."""

    def __init__(self, decomposition: Decomposition | None = None, data=None):
        self.decomposition = decomposition
        self.datavector = None if data is None else np.ascontiguousarray(data, dtype=np.float64)
        self.gammavector = None
        self.thetavector = None
        self.model = None
        self.aic = np.finfo(np.float64).max

    def set_decomposition(self, decomposition: Decomposition):
        self.decomposition = decomposition

    def set_model(self, model):
        self.model = model

    def get_T(self):
        return self.decomposition.get_T()

    def get_R(self):
        return self.decomposition.get_R()

    def get_K(self):
        return self.decomposition.get_K()

    def get_xdim(self):
        return self.decomposition.get_xdim()

    def get_datavector(self):
        return self.datavector

    # data preprocessing (src/petscvector/data/tsdata.cpp:384-560); the model's copy is refreshed
    def _data_changed(self):
        if self.model is not None:
            self.model.problem.set_data(self.datavector)

    def cutdata(self, a: float, b: float):
        """Clamps the data to [a, b] (tsdata.cpp:461-478)."""
        self.datavector = np.minimum(np.maximum(self.datavector, a), b)
        self._data_changed()

    def shiftdata(self, a: float):
        self.datavector = self.datavector + a
        self._data_changed()

    def scaledata(self, a: float, b: float, scale_min: float | None = None, scale_max: float | None = None):
        """Maps [scale_min, scale_max] (default: the data's range) linearly onto [a, b], theta
        with it (tsdata.cpp:384-422, 511-548)."""
        if scale_min is None:
            scale_min, scale_max = float(np.min(self.datavector)), float(np.max(self.datavector))
        self.scale_min, self.scale_max = scale_min, scale_max
        k = (b - a) / (scale_max - scale_min)
        q = a - k * scale_min
        self.datavector = self.datavector * k + q
        self._data_changed()
        if self.model is not None:
            self.model.problem.set_theta(k * self.model.problem.get_theta() + q)

    def unscaledata(self, a: float, b: float):
        """Inverse of scaledata (tsdata.cpp:424-459)."""
        k = (b - a) / (self.scale_max - self.scale_min)
        q = a - k * self.scale_min
        self.datavector = (self.datavector - q) * (1.0 / k)
        self._data_changed()
        if self.model is not None:
            self.model.problem.set_theta((self.model.problem.get_theta() - q) / k)

    def get_gammavector(self):
        if self.model is not None:
            self.gammavector = self.model.problem.get_gamma()
        return self.gammavector

    def get_thetavector(self):
        if self.model is not None:
            self.thetavector = self.model.problem.get_theta()
        return self.thetavector

    def get_aic(self):
        return self.aic

    def set_aic(self, aic):
        self.aic = aic

    def load_gammavector(self, gamma0):
        """TSData::load_gammavector: gamma0 as an array or a PETSc binary file (blocked layout
        as the reference writes it, permuted to the interleaved layout)."""
        if isinstance(gamma0, str):
            from .petscio import load_vec
            gamma0 = load_vec(gamma0)
        self.model.problem.set_gamma(gamma0)
        self.model.problem.permute_gamma()

    def cutgamma(self):
        """Hard assignment: gamma_tk = 1 for the argmax k (true argmax, see the C ABI note)."""
        lab = self.model.problem.argmax_labels()
        nb = self.get_T() * self.get_R()
        g = np.zeros((nb, self.get_K()))
        g[np.arange(nb), lab] = 1.0
        self.model.problem.set_gamma(g.ravel())


class Signal1DData(TSData):
    """Signal1DData<VectorBase>(filename): a 1-D signal (PETSc binary file or array)."""

    def __init__(self, filename_or_data):
        if isinstance(filename_or_data, str):
            from .petscio import load_vec
            data = load_vec(filename_or_data)
        else:
            data = np.ascontiguousarray(filename_or_data, dtype=np.float64)
        super().__init__(None, data)
        self.Tpreliminary = data.size

    def get_Tpreliminary(self):
        return self.Tpreliminary

    def compute_abserr_reconstructed(self, solution) -> float:
        return self.model.problem.abserr_reconstructed(solution)

    def save_signal1d(self, prefix: str):
        """saveSignal1D: <prefix>_gamma.bin (blocked layout) and <prefix>_recovered.bin."""
        from .petscio import save_vec
        T, K = self.get_T(), self.get_K()
        g = self.get_gammavector().reshape(T, K)
        th = self.get_thetavector()
        save_vec(prefix + "_gamma.bin", g.T.ravel())
        save_vec(prefix + "_recovered.bin", g @ th)


class ImageData(TSData):
    """ImageData<VectorBase>(decomposition, filename, width, height): one image (T = 1) or a
    sequence, R = width*height pixels on the decomposition's graph (src/petscvector/data/
    imagedata.cpp:7-38); the file (PETSc binary) or array holds the pixels node-major
    (r*T + t), permuted to the interleaved layout t*R + r."""

    def __init__(self, decomposition: Decomposition, filename_or_data, width: int, height: int):
        if isinstance(filename_or_data, str):
            from .petscio import load_vec
            raw = load_vec(filename_or_data)
        else:
            raw = np.ascontiguousarray(filename_or_data, dtype=np.float64)
        if raw.size != decomposition.get_T() * decomposition.get_R():
            raise PascError(capi.PASC_ERR_ARG, "ImageData: the data does not have T*width*height values")
        self.width, self.height = int(width), int(height)
        super().__init__(decomposition, decomposition.permute_TRxdim(raw))

    def get_width(self):
        return self.width

    def get_height(self):
        return self.height

    def save_image(self, prefix: str, save_original: bool = True):
        """saveImage (imagedata.cpp:40-103): <prefix>_original.bin (the data), _gamma.bin
        (blocked layout) and _recovered.bin (sum_k theta_k gamma_k), pixels node-major."""
        from .petscio import save_vec
        dec = self.decomposition
        if save_original:
            save_vec(prefix + "_original.bin", dec.permute_TRxdim(self.datavector, invert=True))
        g = self.get_gammavector()
        th = self.get_thetavector()
        save_vec(prefix + "_gamma.bin", dec.permute_TRK(g, invert=True))
        rec = g.reshape(-1, self.get_K()) @ th
        save_vec(prefix + "_recovered.bin", dec.permute_TRxdim(rec, invert=True))


class Fem:
    """Fem<VectorBase>(fem_reduce): FEM-SUM temporal coarsening of the gamma step
    (include/general/common/fem.h); fem_reduce = 1 is no reduction."""
    fem_type = 0

    def __init__(self, fem_reduce: float = 1.0):
        self.fem_reduce = float(fem_reduce)

    def is_reduced(self) -> bool:
        return self.fem_reduce < 1.0

    def get_name(self):
        return "FEM-SUM"


class FemHat(Fem):
    """FemHat<VectorBase>(fem_reduce): hat-function coarsening (include/general/common/femhat.h)."""
    fem_type = 1

    def get_name(self):
        return "FEM-HAT"


class GraphH1FEMModel:
    """GraphH1FEMModel<VectorBase>(tsdata, epssqr, fem=None, usethetainpenalty=False).
    Creates the GPU problem; the initial gamma is tsdata's gamma0 (or uniform [0,1) values of
    the given seed, the reference's set_random) in the blocked layout."""

    def __init__(self, tsdata: TSData, epssqr: float, fem=None, usethetainpenalty: bool = False,
                 precision: int = PASC_PREC_MIXED, gamma0=None, seed: int = 13, device: int = 0,
                 gammasolvertype: int = 0):
        self.tsdata = tsdata
        self.epssqr = float(epssqr)
        T, K = tsdata.get_T(), tsdata.get_K()
        graph = tsdata.decomposition.get_graph() if hasattr(tsdata.decomposition, "get_graph") else None
        self.problem = Problem(T, K, epssqr, precision=precision, xdim=tsdata.get_xdim(), device=device, graph=graph)
        T = T * self.problem.R  # blocks of K
        self.fem = fem if fem is not None else Fem(1.0)
        self.problem.set_gamma_solver_type(gammasolvertype)  # graphh1femmodel_gammasolvertype
        if self.fem.is_reduced():
            self.problem.set_fem(self.fem.fem_reduce, self.fem.fem_type)
        self.usethetainpenalty = bool(usethetainpenalty)
        if self.usethetainpenalty:
            self.problem.set_usethetainpenalty(True)
        self.problem.set_data(tsdata.get_datavector())
        if gamma0 is None:
            from .datagen import uniform
            gamma0 = uniform(seed, 0, T * K)
        self.problem.set_gamma(gamma0)
        self.problem.set_theta(np.zeros(K * tsdata.get_xdim()))
        tsdata.set_model(self)

    def set_epssqr(self, epssqr: float):
        self.epssqr = float(epssqr)
        self.problem.set_epssqr(epssqr)

    def get_aic(self, L: float) -> float:
        return 2 * np.log(L) + self.tsdata.get_K()

    def get_usethetainpenalty(self) -> bool:
        return self.usethetainpenalty

    def get_name(self):
        return "Graph-H1-FEM Time-Series Model"

    def get_epssqr(self) -> float:
        return self.epssqr

    def get_T(self) -> int:
        """Timesteps of the data (GraphH1FEMModel::get_T, graphh1fem.h:461-463)."""
        return self.tsdata.get_T()

    def get_T_reduced(self) -> int:
        """Timesteps of the gamma QP: ceil(T*fem_reduce) under FEM coarsening, else T
        (graphh1fem.h:456-458)."""
        return self.problem.get_fem()[2] if self.fem.is_reduced() else self.tsdata.get_T()

    def get_fem_reduce(self) -> float:
        return self.fem.fem_reduce

    def get_graph(self):
        """The decomposition's graph (None for a 1-D signal)."""
        d = self.tsdata.decomposition
        return d.get_graph() if hasattr(d, "get_graph") else None

    def get_L(self, gammasolver=None, thetasolver=None) -> float:
        """The gamma QP's objective at the current gamma and theta (GraphH1FEMModel::get_L
        returns the gamma solver's fx, graphh1fem.h:366-370)."""
        return self.problem.get_fx()

    def get_linear_quadratic(self, gammasolver=None, thetasolver=None):
        """(0, 0), as GraphH1FEMModel::get_linear_quadratic sets both (graphh1fem.h:373-377)."""
        return 0.0, 0.0


class SPGQPSolver:
    """SPGQPSolver<VectorBase> on the model's QP (gamma step)."""

    def __init__(self, model: GraphH1FEMModel, options: dict | None = None):
        self.model = model
        self.opts = spg_opts_from(options)
        self.it_sum = 0
        self.hessmult_sum = 0
        self.last: SpgqpStats | None = None

    def solve(self):
        self.last = self.model.problem.spgqp_solve(self.opts)
        self.it_sum += self.last.it
        self.hessmult_sum += self.last.hessmult

    def get_fx(self) -> float:
        return self.model.problem.get_fx()

    def get_it(self) -> int:
        return self.it_sum

    def get_hessmult(self) -> int:
        return self.hessmult_sum


class TSSolver:
    """TSSolver<VectorBase>(tsdata, annealing): the alternating theta/gamma loop."""

    def __init__(self, tsdata: TSData, annealing: int = 1, options: dict | None = None):
        self.tsdata = tsdata
        self.model = tsdata.model
        self.annealing = int(annealing)
        self.options = dict(options or {})
        self.gammasolver = SPGQPSolver(self.model, self.options)
        self.thetasolved = False
        self.L = np.finfo(np.float64).max
        self.stats: TsStats | None = None

    def set_solution_theta(self, theta):
        self.model.problem.set_theta(theta)
        self.thetasolved = True

    def set_annealing(self, annealing: int):
        self.annealing = int(annealing)

    def solve(self, gamma_restart=None):
        ts = ts_opts_from(self.options)
        ts.annealing = self.annealing
        ts.thetasolved = 1 if self.thetasolved else 0
        self.stats = self.model.problem.ts_solve(ts, self.gammasolver.opts, gamma_restart)
        self.L = self.stats.L
        self.gammasolver.it_sum += self.stats.spg_it_sum
        self.tsdata.set_aic(self.stats.aic)
        return self.stats

    def get_L(self) -> float:
        return self.L

    def get_gammasolver(self) -> SPGQPSolver:
        return self.gammasolver
