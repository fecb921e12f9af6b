"""ctypes wrapper of the FP64 CPU oracle (oracle/pasc_oracle.c) and of the reference-compiled
library (oracle/_ref/libpasc_ref.so, present only where the reference tree was available).

TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
import this module; the GPU library never uses it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpasc_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libpasc_ref.so")

_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


class SpgOpts(C.Structure):
    """pasc_oracle_spg_opts (defaults: include/general/solver/spgqpsolver.h:19-36)."""

    _fields_ = [
        ("maxit", C.c_int), ("eps", C.c_double), ("m", C.c_int), ("gamma", C.c_double),
        ("sigma1", C.c_double), ("sigma2", C.c_double), ("alphainit", C.c_double),
        ("stop_difff", C.c_int), ("stop_normgp", C.c_int), ("stop_normgp_normb", C.c_int),
        ("stop_Anormgp", C.c_int), ("stop_Anormgp_normb", C.c_int),
    ]


class SpgResult(C.Structure):
    _fields_ = [("it", C.c_int), ("hessmult", C.c_int), ("fx", C.c_double),
                ("gP", C.c_double), ("dAd", C.c_double), ("normb", C.c_double)]


class TsOpts(C.Structure):
    """pasc_oracle_ts_opts (defaults: include/general/solver/tssolver.h:13-15)."""

    _fields_ = [("maxit", C.c_int), ("eps", C.c_double), ("init_permute", C.c_int),
                ("annealing", C.c_int), ("relative", C.c_int), ("thetasolved", C.c_int)]


class TsResult(C.Structure):
    _fields_ = [("it_last", C.c_int), ("it_sum", C.c_int), ("spg_it_sum", C.c_int),
                ("spg_hessmult_sum", C.c_int), ("L", C.c_double), ("deltaL", C.c_double),
                ("aic", C.c_double), ("L_increased", C.c_int)]


def build(force: bool = False) -> str:
    """Compile oracle/pasc_oracle.c into oracle/libpasc_oracle.so (gcc, OpenMP, no FMA)."""
    src = os.path.join(HERE, "pasc_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call([
            os.environ.get("CC", "gcc"), "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off",
            "-fPIC", "-shared", "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


REF_FLAT_PATH = os.path.join(HERE, "_ref", "libpasc_ref_flat.cpp")


def build_ref() -> str | None:
    """Compile the reference's own solver templates: from the reference tree where it is
    (build_ref.sh), else from the single translation unit that recipe wrote into oracle/_ref
    (a machine without the tree, given a copy of this checkout); None if neither exists."""
    script = os.path.join(HERE, "build_ref.sh")
    subprocess.check_call(["sh", script])
    if not os.path.exists(REF_LIB_PATH) and os.path.exists(REF_FLAT_PATH):
        subprocess.check_call([os.environ.get("CXX", "g++"), "-std=c++14", "-O2", "-fopenmp", "-fPIC", "-shared",
                               "-ffp-contract=off", "-w", REF_FLAT_PATH, "-o", REF_LIB_PATH])
    return REF_LIB_PATH if os.path.exists(REF_LIB_PATH) else None


class AdjOpts(C.Structure):
    _fields_ = [("act_tol", C.c_double), ("cg_tol", C.c_double), ("cg_maxit", C.c_int)]


class AdjResult(C.Structure):
    _fields_ = [("cg_it", C.c_int), ("status", C.c_int), ("free_dims", C.c_long), ("cg_relres", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.pasc_oracle_spg_default_opts.argtypes = [C.POINTER(SpgOpts)]
        L.pasc_oracle_ts_default_opts.argtypes = [C.POINTER(TsOpts)]
        L.pasc_oracle_project.argtypes = [_dp, C.c_long, C.c_int, C.c_int]
        L.pasc_oracle_fem_h1_matmult.argtypes = [_dp, _dp, C.c_long, C.c_int, C.c_double, C.c_int]
        L.pasc_oracle_residual_b.argtypes = [_dp, _dp, _dp, C.c_long, C.c_int, C.c_int, C.c_double, C.c_int]
        L.pasc_oracle_theta_update.argtypes = [_dp, _dp, _dp, C.c_long, C.c_int, C.c_int, C.c_int]
        L.pasc_oracle_permute_blocked_to_interleaved.argtypes = [_dp, _dp, C.c_long, C.c_int]
        L.pasc_oracle_A_coeff.argtypes = [C.c_double, C.c_long, C.c_int]
        L.pasc_oracle_A_coeff.restype = C.c_double
        L.pasc_oracle_b_coeff.argtypes = [C.c_long, C.c_int]
        L.pasc_oracle_b_coeff.restype = C.c_double
        L.pasc_oracle_spgqp_solve.argtypes = [_dp, _dp, C.c_long, C.c_int, C.c_double,
                                              C.POINTER(SpgOpts), C.POINTER(SpgResult),
                                              C.c_void_p, C.c_int]
        L.pasc_oracle_tssolver_solve.argtypes = [_dp, _dp, _dp, C.c_long, C.c_int, C.c_int,
                                                 C.c_double, C.c_int, C.POINTER(TsOpts),
                                                 C.POINTER(SpgOpts), C.c_void_p,
                                                 C.POINTER(TsResult), C.c_void_p, C.c_int]
        L.pasc_oracle_abserr_reconstructed.argtypes = [_dp, _dp, _dp, C.c_long, C.c_int]
        L.pasc_oracle_abserr_reconstructed.restype = C.c_double
        L.pasc_oracle_argmax_labels.argtypes = [_dp, _ip, C.c_long, C.c_int]
        L.pasc_oracle_fem_T_reduced.argtypes = [C.c_long, C.c_double]
        L.pasc_oracle_fem_T_reduced.restype = C.c_long
        L.pasc_oracle_fem_reduce.argtypes = [_dp, _dp, C.c_long, C.c_long, C.c_int, C.c_int]
        L.pasc_oracle_fem_prolongate.argtypes = [_dp, _dp, C.c_long, C.c_long, C.c_int, C.c_int]
        L.pasc_oracle_tssolver_solve_fem.argtypes = [_dp, _dp, _dp, C.c_long, C.c_int, C.c_double, C.c_int,
                                                     C.c_double, C.c_int, C.POINTER(TsOpts), C.POINTER(SpgOpts),
                                                     C.POINTER(TsResult), C.c_int]
        L.pasc_oracle_graph_matmult.argtypes = [_dp, _dp, C.c_long, C.c_int, C.c_double, C.POINTER(Graph), C.c_int]
        L.pasc_oracle_spgqp_solve_graph.argtypes = [_dp, _dp, C.c_long, C.c_int, C.c_double, C.POINTER(Graph),
                                                    C.POINTER(SpgOpts), C.POINTER(SpgResult), C.c_int]
        L.pasc_oracle_permute_TRK.argtypes = [_dp, _dp, C.c_long, C.c_long, C.c_int]
        L.pasc_oracle_graph_grid1d.argtypes = [C.c_int, _ip, _ip]
        L.pasc_oracle_graph_grid2d.argtypes = [C.c_int, C.c_int, _ip, _ip]
        L.pasc_oracle_graph_threshold.argtypes = [_dp, C.c_int, C.c_int, C.c_double, _ip, C.c_void_p]
        L.pasc_oracle_graph_threshold.restype = C.c_long
        L.pasc_oracle_tssolver_solve_graph.argtypes = [_dp, _dp, _dp, C.c_long, C.c_int, C.c_double, C.c_int,
                                                       C.POINTER(Graph), C.POINTER(TsOpts), C.POINTER(SpgOpts),
                                                       C.POINTER(TsResult), C.c_int]
        L.pasc_oracle_spgqp_solve_coeff.argtypes = [_dp, _dp, C.c_long, C.c_int, C.c_double, C.c_void_p,
                                                    C.POINTER(SpgOpts), C.POINTER(SpgResult), C.c_int]
        L.pasc_oracle_tssolver_solve_coeff.argtypes = [_dp, _dp, _dp, C.c_long, C.c_int, C.c_double, C.c_int,
                                                       C.c_void_p, C.POINTER(TsOpts), C.POINTER(SpgOpts),
                                                       C.POINTER(TsResult), C.c_int]
        L.pasc_oracle_fem_h1_matmult_kc.argtypes = [_dp, _dp, C.c_long, C.c_int, _dp, C.c_int]
        L.pasc_oracle_spgqp_solve_kc.argtypes = [_dp, _dp, C.c_long, C.c_int, _dp, C.POINTER(SpgOpts),
                                                 C.POINTER(SpgResult), C.c_int]
        L.pasc_oracle_theta_update_penalty.argtypes = [_dp, _dp, _dp, C.c_long, C.c_int, C.c_double]
        L.pasc_oracle_tssolver_solve_model.argtypes = [_dp, _dp, _dp, C.c_long, C.c_int, C.c_double, C.c_int,
                                                       C.c_double, C.c_int, C.c_int, C.POINTER(TsOpts),
                                                       C.POINTER(SpgOpts), C.POINTER(TsResult), C.c_int]
        L.pasc_oracle_recon_mse.argtypes = [_dp, _dp, _dp, C.c_long, C.c_int, C.c_void_p, C.c_void_p]
        L.pasc_oracle_recon_mse.restype = C.c_double
        L.pasc_oracle_adjoint.argtypes = [_dp, _dp, _dp, _dp, C.c_long, C.c_int, C.c_double, C.c_double,
                                          C.c_double, C.POINTER(AdjOpts), C.c_void_p, C.POINTER(C.c_double),
                                          C.c_void_p, C.c_void_p, C.POINTER(AdjResult)]
        _lib = L
    return _lib


def spg_opts(**kw) -> SpgOpts:
    o = SpgOpts()
    lib().pasc_oracle_spg_default_opts(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def ts_opts(**kw) -> TsOpts:
    o = TsOpts()
    lib().pasc_oracle_ts_default_opts(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def project(x, T, K, nthreads=1):
    y = _f64(x).copy()
    lib().pasc_oracle_project(y, T, K, nthreads)
    return y


def matmult(x, T, K, coeff, nthreads=1):
    x = _f64(x)
    y = np.empty_like(x)
    lib().pasc_oracle_fem_h1_matmult(x, y, T, K, coeff, nthreads)
    return y


def A_coeff(epssqr, T, scalef=1):
    return lib().pasc_oracle_A_coeff(epssqr, T, scalef)


def b_coeff(T, scalef=1):
    return lib().pasc_oracle_b_coeff(T, scalef)


def residual_b(data, theta, T, K, xdim=1, bscale=None, nthreads=1):
    if bscale is None:
        bscale = b_coeff(T)
    b = np.empty(T * K)
    lib().pasc_oracle_residual_b(_f64(data), _f64(theta), b, T, K, xdim, bscale, nthreads)
    return b


def theta_update(gamma, data, T, K, xdim=1, nthreads=1):
    th = np.empty(K * xdim)
    lib().pasc_oracle_theta_update(_f64(gamma), _f64(data), th, T, K, xdim, nthreads)
    return th


def permute_blocked_to_interleaved(v, T, K):
    out = np.empty(T * K)
    lib().pasc_oracle_permute_blocked_to_interleaved(_f64(v), out, T, K)
    return out


def spgqp_solve(b, x0, T, K, coeff, opts: SpgOpts | None = None, trace=False, nthreads=1):
    """Returns (x, SpgResult, trace array [it+1, 8] or None)."""
    opts = opts or spg_opts()
    x = _f64(x0).copy()
    r = SpgResult()
    tr = np.zeros((opts.maxit + 1) * 8) if trace else None
    lib().pasc_oracle_spgqp_solve(_f64(b), x, T, K, coeff, C.byref(opts), C.byref(r),
                                  tr.ctypes.data if trace else None, nthreads)
    if trace:
        tr = tr.reshape(-1, 8)[: r.it + 1].copy()
    return x, r, tr


def tssolver_solve(data, gamma_raw, theta0, T, K, epssqr, xdim=1, scalef=1,
                   ts: TsOpts | None = None, spg: SpgOpts | None = None,
                   gamma_restart=None, nthreads=1):
    """Returns (gamma, theta, TsResult, trace_L)."""
    ts = ts or ts_opts()
    spg = spg or spg_opts()
    g = _f64(gamma_raw).copy()
    th = _f64(theta0).copy()
    r = TsResult()
    nL = ts.maxit * max(1, ts.annealing)
    trL = np.full(nL, np.nan)
    gr = _f64(gamma_restart) if gamma_restart is not None else None
    lib().pasc_oracle_tssolver_solve(_f64(data), g, th, T, K, xdim, epssqr, scalef,
                                     C.byref(ts), C.byref(spg),
                                     gr.ctypes.data if gr is not None else None,
                                     C.byref(r), trL.ctypes.data, nthreads)
    return g, th, r, trL[~np.isnan(trL)]


def abserr_reconstructed(gamma, theta, solution, T, K):
    return lib().pasc_oracle_abserr_reconstructed(_f64(gamma), _f64(theta), _f64(solution), T, K)


def argmax_labels(gamma, T, K):
    lab = np.empty(T, dtype=np.int32)
    lib().pasc_oracle_argmax_labels(_f64(gamma), lab, T, K)
    return lab


def fem_T_reduced(T, fem_reduce):
    return lib().pasc_oracle_fem_T_reduced(T, fem_reduce)


def fem_reduce(g1, T1, T2, K, fem_type=0):
    g2 = np.empty(T2 * K)
    lib().pasc_oracle_fem_reduce(_f64(g1), g2, T1, T2, K, fem_type)
    return g2


def fem_prolongate(g2, T1, T2, K, fem_type=0):
    g1 = np.empty(T1 * K)
    lib().pasc_oracle_fem_prolongate(_f64(g2), g1, T1, T2, K, fem_type)
    return g1


def tssolver_solve_fem(data, gamma_raw, theta0, T, K, epssqr, fem_reduce, fem_type=0, scalef=1,
                       ts: TsOpts | None = None, spg: SpgOpts | None = None, nthreads=1):
    """Returns (gamma, theta, TsResult)."""
    ts = ts or ts_opts()
    spg = spg or spg_opts()
    g = _f64(gamma_raw).copy()
    th = _f64(theta0).copy()
    r = TsResult()
    lib().pasc_oracle_tssolver_solve_fem(_f64(data), g, th, T, K, epssqr, scalef, fem_reduce, fem_type,
                                         C.byref(ts), C.byref(spg), C.byref(r), nthreads)
    return g, th, r


def theta_update_penalty(gamma, data, T, K, alpha):
    th = np.empty(K)
    lib().pasc_oracle_theta_update_penalty(_f64(gamma), _f64(data), th, T, K, alpha)
    return th


def fem_h1_matmult_kc(x, T, K, kc):
    y = np.empty(T * K)
    lib().pasc_oracle_fem_h1_matmult_kc(_f64(x), y, T, K, _f64(kc), 1)
    return y


def spgqp_solve_kc(b, x0, T, K, kc, opts: SpgOpts | None = None):
    opts = opts or spg_opts()
    x = _f64(x0).copy()
    r = SpgResult()
    lib().pasc_oracle_spgqp_solve_kc(_f64(b), x, T, K, _f64(kc), C.byref(opts), C.byref(r), 1)
    return x, r


def tssolver_solve_model(data, gamma_raw, theta0, T, K, epssqr, fem_reduce=1.0, fem_type=0,
                         usethetainpenalty=False, scalef=1, ts: TsOpts | None = None,
                         spg: SpgOpts | None = None, nthreads=1):
    """Returns (gamma, theta, TsResult)."""
    ts = ts or ts_opts()
    spg = spg or spg_opts()
    g = _f64(gamma_raw).copy()
    th = _f64(theta0).copy()
    r = TsResult()
    rc = lib().pasc_oracle_tssolver_solve_model(_f64(data), g, th, T, K, epssqr, scalef, fem_reduce, fem_type,
                                                1 if usethetainpenalty else 0, C.byref(ts), C.byref(spg),
                                                C.byref(r), nthreads)
    if rc != 0:
        raise ValueError("tssolver_solve_model: unsupported combination")
    return g, th, r


class Graph(C.Structure):
    """pasc_oracle_graph: CSR neighbour lists of R nodes (sorted, no self, no duplicates)."""

    _fields_ = [("R", C.c_long), ("ptr", C.POINTER(C.c_int)), ("idx", C.POINTER(C.c_int))]


def make_graph(ptr, idx):
    """(Graph structure, the arrays it points into) -- keep both alive together."""
    ptr = np.ascontiguousarray(ptr, dtype=np.int32)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    if idx.size == 0:
        idx = np.zeros(1, dtype=np.int32)
    g = Graph(len(ptr) - 1, ptr.ctypes.data_as(C.POINTER(C.c_int)), idx.ctypes.data_as(C.POINTER(C.c_int)))
    return g, (ptr, idx)


def graph_grid1d(width):
    ptr = np.empty(width + 1, dtype=np.int32)
    idx = np.empty(max(2 * (width - 1), 1), dtype=np.int32)
    lib().pasc_oracle_graph_grid1d(width, ptr, idx)
    return ptr, idx[: ptr[-1]].copy()


def graph_grid2d(width, height):
    ptr = np.empty(width * height + 1, dtype=np.int32)
    idx = np.empty(max(2 * (height * (width - 1) + width * (height - 1)), 1), dtype=np.int32)
    lib().pasc_oracle_graph_grid2d(width, height, ptr, idx)
    return ptr, idx[: ptr[-1]].copy()


def graph_threshold(coords, n, dim, threshold):
    """coords: dim*n values, dimension by dimension (c[i + d*n])."""
    c = _f64(coords)
    ptr = np.empty(n + 1, dtype=np.int32)
    nnz = lib().pasc_oracle_graph_threshold(c, n, dim, threshold, ptr, None)
    idx = np.empty(max(nnz, 1), dtype=np.int32)
    lib().pasc_oracle_graph_threshold(c, n, dim, threshold, ptr, idx.ctypes.data)
    return ptr, idx[:nnz].copy()


def graph_matmult(x, T, K, coeff, ptr, idx):
    g, keep = make_graph(ptr, idx)
    y = np.empty(T * g.R * K)
    lib().pasc_oracle_graph_matmult(_f64(x), y, T, K, coeff, C.byref(g), 1)
    return y


def spgqp_solve_graph(b, x0, T, K, coeff, ptr, idx, opts: SpgOpts | None = None):
    opts = opts or spg_opts()
    g, keep = make_graph(ptr, idx)
    x = _f64(x0).copy()
    r = SpgResult()
    lib().pasc_oracle_spgqp_solve_graph(_f64(b), x, T, K, coeff, C.byref(g), C.byref(opts), C.byref(r), 1)
    return x, r


def permute_TRK(v, T, R, K):
    out = np.empty(T * R * K)
    lib().pasc_oracle_permute_TRK(_f64(v), out, T, R, K)
    return out


def tssolver_solve_graph(data, gamma_raw, theta0, T, K, epssqr, ptr, idx, scalef=1, ts: TsOpts | None = None,
                         spg: SpgOpts | None = None, nthreads=1):
    """Returns (gamma, theta, TsResult); data T*R, gamma T*R*K (blocked when ts.init_permute)."""
    ts = ts or ts_opts()
    spg = spg or spg_opts()
    gr, keep = make_graph(ptr, idx)
    g = _f64(gamma_raw).copy()
    th = _f64(theta0).copy()
    r = TsResult()
    rc = lib().pasc_oracle_tssolver_solve_graph(_f64(data), g, th, T, K, epssqr, scalef, C.byref(gr), C.byref(ts),
                                                C.byref(spg), C.byref(r), nthreads)
    if rc != 0:
        raise MemoryError("tssolver_solve_graph")
    return g, th, r


def spgqp_solve_coeff(b, x0, T, K, coeff, opts: SpgOpts | None = None, ptr=None, idx=None):
    """SPGQPSolverC; with ptr/idx on the graph of those neighbour lists."""
    opts = opts or spg_opts()
    x = _f64(x0).copy()
    r = SpgResult()
    if ptr is not None:
        g, keep = make_graph(ptr, idx)
        gp = C.cast(C.pointer(g), C.c_void_p)
    else:
        gp = None
    lib().pasc_oracle_spgqp_solve_coeff(_f64(b), x, T, K, coeff, gp, C.byref(opts), C.byref(r), 1)
    return x, r


def tssolver_solve_coeff(data, gamma_raw, theta0, T, K, epssqr, ptr=None, idx=None, scalef=1,
                         ts: TsOpts | None = None, spg: SpgOpts | None = None, nthreads=1):
    ts = ts or ts_opts()
    spg = spg or spg_opts()
    if ptr is not None:
        gr, keep = make_graph(ptr, idx)
        gp = C.cast(C.pointer(gr), C.c_void_p)
    else:
        gp = None
    g = _f64(gamma_raw).copy()
    th = _f64(theta0).copy()
    r = TsResult()
    rc = lib().pasc_oracle_tssolver_solve_coeff(_f64(data), g, th, T, K, epssqr, scalef, gp, C.byref(ts),
                                                C.byref(spg), C.byref(r), nthreads)
    if rc != 0:
        raise MemoryError("tssolver_solve_coeff")
    return g, th, r


def recon_mse(gamma, theta, clean, T, K):
    """Returns (loss, dloss/dgamma [N], direct dloss/dtheta [K])."""
    dg = np.empty(T * K)
    dth = np.empty(K)
    loss = lib().pasc_oracle_recon_mse(_f64(gamma), _f64(theta), _f64(clean), T, K, dg.ctypes.data,
                                       dth.ctypes.data)
    return loss, dg, dth


def adjoint(gamma, data, theta, dloss_dgamma, T, K, epssqr, scalef=1, act_tol=1e-7, cg_tol=1e-10,
            cg_maxit=20000):
    """Returns (dloss/d epssqr, dloss/d data [T], dloss/d theta [K] (through b only), lambda [N],
    AdjResult)."""
    o = AdjOpts(act_tol=act_tol, cg_tol=cg_tol, cg_maxit=cg_maxit)
    r = AdjResult()
    lam = np.empty(T * K)
    dX = np.empty(T)
    dth = np.empty(K)
    deps = C.c_double()
    coeff = A_coeff(epssqr, T, scalef)
    dcoeff = (1.0 / T) if scalef else 1.0
    lib().pasc_oracle_adjoint(_f64(gamma), _f64(data), _f64(theta), _f64(dloss_dgamma), T, K, coeff, dcoeff,
                              b_coeff(T, scalef), C.byref(o), lam.ctypes.data, C.byref(deps), dX.ctypes.data,
                              dth.ctypes.data, C.byref(r))
    return deps.value, dX, dth, lam, r


# --------------------------------------------------------------------------------------
# reference-compiled library (oracle/_ref); available only where the reference tree is
# --------------------------------------------------------------------------------------
_ref = None


def ref_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_LIB_PATH)
        R.ref_set_option.argtypes = [C.c_char_p, C.c_double]
        R.ref_set_threads.argtypes = [C.c_int]
        R.ref_project.argtypes = [_dp, C.c_int, C.c_int]
        R.ref_fs_sequence.argtypes = [C.c_int, _dp, C.c_int, _dp]
        R.ref_matmult.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_double]
        R.ref_spgqp_solve.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_double, _dp]
        R.ref_tssolver_solve.argtypes = [_dp, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double,
                                         C.c_int, C.c_int, _dp, _dp]
        _ref = R
    return _ref


def ref_options(nthreads=1, **kw):
    """Sets the reference's console options for the next call and the threads of its host-array
    backend (1: sequential sums in index order; n > 1: the oracle's chunked order for n, 0: all
    cores)."""
    R = ref()
    R.ref_set_threads(int(nthreads))
    R.ref_clear_options()
    for k, v in kw.items():
        R.ref_set_option(k.encode(), float(v))


def ref_project(x, T, K):
    y = _f64(x).copy()
    ref().ref_project(y, T, K)
    return y


def ref_matmult(x, T, K, coeff):
    x = _f64(x)
    y = np.empty_like(x)
    ref().ref_matmult(x, y, T, K, coeff)
    return y


def ref_fs_sequence(m, values):
    v = _f64(values)
    out = np.empty_like(v)
    ref().ref_fs_sequence(m, v, len(v), out)
    return out


def ref_spgqp_solve(b, x0, T, K, coeff, nthreads=1, **options):
    ref_options(nthreads, **options)
    x = _f64(x0).copy()
    out = np.zeros(3)
    ref().ref_spgqp_solve(_f64(b), x, T, K, coeff, out)
    return x, int(out[0]), int(out[1]), float(out[2])


def ref_tssolver_solve(data, gamma_random, theta0, T, K, epssqr, xdim=1, annealing=1,
                       theta_given=False, **options):
    ref_options(**options)
    th = _f64(theta0).copy()
    g = np.zeros(T * K)
    out = np.zeros(4)
    ref().ref_tssolver_solve(_f64(data), _f64(gamma_random), th, T, K, xdim, epssqr,
                             annealing, 1 if theta_given else 0, g, out)
    return g, th, dict(L=out[0], it_last=int(out[1]), it_sum=int(out[2]), aic=out[3])
