"""ctypes binding of the C ABI in include/pasc_gb300.h.

This is the binding a Python caller of the reference's path would add: every function of
the header with its argument types.  Loading fails loudly when libpasc_gb300.so has not
been built (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libpasc_gb300.so")

PASC_OK = 0
PASC_ERR_ARG, PASC_ERR_CUDA, PASC_ERR_ALLOC, PASC_ERR_STATE, PASC_ERR_NOTSUPP, PASC_ERR_TIMEOUT = 1, 2, 3, 4, 5, 6
PASC_SPG_RUNNING, PASC_SPG_CONVERGED, PASC_SPG_MAXIT, PASC_SPG_DAD_ZERO, PASC_SPG_NONFINITE = 0, 1, 2, 3, 4
PASC_PREC_FP64, PASC_PREC_MIXED = 0, 1

STATUS_NAMES = {0: "running", 1: "converged", 2: "maxit", 3: "dAd_zero", 4: "nonfinite"}


class SpgqpOpts(C.Structure):
    _fields_ = [
        ("maxit", C.c_int), ("eps", C.c_double), ("m", C.c_int), ("gamma", C.c_double),
        ("sigma1", C.c_double), ("sigma2", C.c_double), ("alphainit", C.c_double),
        ("stop_difff", C.c_int), ("stop_normgp", C.c_int), ("stop_normgp_normb", C.c_int),
        ("stop_Anormgp", C.c_int), ("stop_Anormgp_normb", C.c_int),
    ]


class SpgqpStats(C.Structure):
    _fields_ = [("it", C.c_int), ("hessmult", C.c_int), ("status", C.c_int),
                ("kernel_launches", C.c_int), ("fx", C.c_double), ("gP", C.c_double),
                ("dAd", C.c_double), ("time_s", C.c_double)]


class TsOpts(C.Structure):
    _fields_ = [("maxit", C.c_int), ("eps", C.c_double), ("init_permute", C.c_int),
                ("annealing", C.c_int), ("relative", C.c_int), ("thetasolved", C.c_int)]


class TsStats(C.Structure):
    _fields_ = [("it_last", C.c_int), ("it_sum", C.c_int), ("spg_it_sum", C.c_int),
                ("spg_hessmult_sum", C.c_int), ("kernel_launches", C.c_int),
                ("L_increased", C.c_int), ("L", C.c_double), ("deltaL", C.c_double),
                ("aic", C.c_double), ("time_s", C.c_double)]


class AdjointOpts(C.Structure):
    _fields_ = [("act_tol", C.c_double), ("cg_tol", C.c_double), ("cg_maxit", C.c_int)]


class AdjointStats(C.Structure):
    _fields_ = [("cg_it", C.c_int), ("status", C.c_int), ("kernel_launches", C.c_int),
                ("free_dims", C.c_long), ("cg_relres", C.c_double), ("time_s", C.c_double)]


class PolishOpts(C.Structure):
    _fields_ = [("rounds", C.c_int), ("act_tol", C.c_double), ("cg_tol", C.c_double), ("cg_maxit", C.c_int)]


class PolishStats(C.Structure):
    _fields_ = [("rounds", C.c_int), ("cg_it", C.c_int), ("kernel_launches", C.c_int),
                ("face_changes", C.c_long), ("cg_status", C.c_int), ("cg_relres", C.c_double),
                ("step_rel", C.c_double), ("fx", C.c_double), ("time_s", C.c_double)]


class PascError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pasc_gb300 error {code}: {msg}")
        self.code = code


_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
LONG_DTYPE = np.int64 if C.sizeof(C.c_long) == 8 else np.int32
_lp = np.ctypeslib.ndpointer(LONG_DTYPE, flags="C_CONTIGUOUS")
_h = C.c_void_p

# name -> (restype, argtypes); the complete list of exported symbols of include/pasc_gb300.h
PROTOTYPES = {
    "pasc_gb300_spgqp_default_opts": (None, [C.POINTER(SpgqpOpts)]),
    "pasc_gb300_ts_default_opts": (None, [C.POINTER(TsOpts)]),
    "pasc_gb300_abi_version": (C.c_int, []),
    "pasc_gb300_last_error": (C.c_char_p, []),
    "pasc_gb300_device_count": (C.c_int, []),
    "pasc_gb300_create": (C.c_int, [C.POINTER(_h), C.c_long, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int]),
    "pasc_gb300_destroy": (C.c_int, [_h]),
    "pasc_gb300_set_epssqr": (C.c_int, [_h, C.c_double, C.c_int]),
    "pasc_gb300_set_data": (C.c_int, [_h, _dp]),
    "pasc_gb300_set_gamma": (C.c_int, [_h, _dp]),
    "pasc_gb300_get_gamma": (C.c_int, [_h, _dp]),
    "pasc_gb300_set_data_f32": (C.c_int, [_h, _fp]),
    "pasc_gb300_set_gamma_f32": (C.c_int, [_h, _fp]),
    "pasc_gb300_get_gamma_f32": (C.c_int, [_h, _fp]),
    "pasc_gb300_host_alloc": (C.c_int, [C.POINTER(C.c_void_p), C.c_ulong]),
    "pasc_gb300_host_free": (C.c_int, [C.c_void_p]),
    "pasc_gb300_set_theta": (C.c_int, [_h, _dp]),
    "pasc_gb300_get_theta": (C.c_int, [_h, _dp]),
    "pasc_gb300_permute_gamma": (C.c_int, [_h]),
    "pasc_gb300_update_theta": (C.c_int, [_h]),
    "pasc_gb300_update_b": (C.c_int, [_h]),
    "pasc_gb300_spgqp_solve": (C.c_int, [_h, C.POINTER(SpgqpOpts), C.POINTER(SpgqpStats)]),
    "pasc_gb300_spgqp_start": (C.c_int, [_h, C.POINTER(SpgqpOpts)]),
    "pasc_gb300_spgqp_iterate": (C.c_int, [_h, C.c_long, C.c_int, C.POINTER(SpgqpStats)]),
    "pasc_gb300_spgqp_last_iterate": (C.c_int, [_h, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "pasc_gb300_set_sweep_variant": (C.c_int, [_h, C.c_int]),
    "pasc_gb300_get_sweep_variant": (C.c_int, [_h, C.POINTER(C.c_int)]),
    "pasc_gb300_get_sweep_tuning": (C.c_int, [_h, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "pasc_gb300_get_b": (C.c_int, [_h, _dp]),
    "pasc_gb300_set_fem": (C.c_int, [_h, C.c_double, C.c_int]),
    "pasc_gb300_get_fem": (C.c_int, [_h, C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_long)]),
    "pasc_gb300_fem_reduce_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_long, C.c_int, C.c_int, C.c_void_p]),
    "pasc_gb300_fem_prolongate_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_long, C.c_int, C.c_int,
                                                C.c_void_p]),
    "pasc_gb300_create_graph": (C.c_int, [C.POINTER(_h), C.c_long, C.c_long, C.c_int, C.c_int, C.c_double, C.c_int,
                                          _ip, _ip]),
    "pasc_gb300_get_graph": (C.c_int, [_h, C.POINTER(C.c_long), C.POINTER(C.c_long), C.POINTER(C.c_long)]),
    "pasc_gb300_graph_grid1d": (C.c_int, [C.c_int, _ip, _ip]),
    "pasc_gb300_graph_grid2d": (C.c_int, [C.c_int, C.c_int, _ip, _ip]),
    "pasc_gb300_graph_threshold": (C.c_int, [_dp, C.c_int, C.c_int, C.c_double, _ip, C.c_void_p, C.c_long,
                                             C.POINTER(C.c_long)]),
    "pasc_gb300_graph_matmult_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_long, C.c_int, C.c_double,
                                               C.c_void_p, C.c_void_p, C.c_void_p]),
    "pasc_gb300_set_gamma_solver_type": (C.c_int, [_h, C.c_int]),
    "pasc_gb300_get_gamma_solver_type": (C.c_int, [_h, C.POINTER(C.c_int)]),
    "pasc_gb300_set_usethetainpenalty": (C.c_int, [_h, C.c_int]),
    "pasc_gb300_get_usethetainpenalty": (C.c_int, [_h, C.POINTER(C.c_int)]),
    "pasc_gb300_time_model_kernels": (C.c_int, [_h, C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "pasc_gb300_set_residual_engine": (C.c_int, [_h, C.c_int]),
    "pasc_gb300_get_residual_engine": (C.c_int, [_h, C.POINTER(C.c_int)]),
    "pasc_gb300_get_fx": (C.c_int, [_h, C.POINTER(C.c_double)]),
    "pasc_gb300_ts_solve": (C.c_int, [_h, C.POINTER(TsOpts), C.POINTER(SpgqpOpts), C.c_void_p,
                                      C.POINTER(TsStats)]),
    "pasc_gb300_abserr_reconstructed": (C.c_int, [_h, _dp, C.POINTER(C.c_double)]),
    "pasc_gb300_argmax_labels": (C.c_int, [_h, _ip]),
    "pasc_gb300_project_f64": (C.c_int, [C.c_void_p, C.c_long, C.c_int, C.c_void_p]),
    "pasc_gb300_project_f32": (C.c_int, [C.c_void_p, C.c_long, C.c_int, C.c_void_p]),
    "pasc_gb300_fem_h1_matmult_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_int, C.c_double,
                                                C.c_void_p]),
    "pasc_gb300_fem_h1_matmult_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_int, C.c_float,
                                                C.c_void_p]),
    "pasc_gb300_theta_update_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_int, C.c_void_p,
                                                  C.c_void_p]),
    "pasc_gb300_vec_alloc": (C.c_int, [C.POINTER(C.c_void_p), C.c_long, C.c_int]),
    "pasc_gb300_vec_free": (C.c_int, [C.c_void_p]),
    "pasc_gb300_vec_set": (C.c_int, [C.c_void_p, _dp, C.c_long]),
    "pasc_gb300_vec_get": (C.c_int, [C.c_void_p, _dp, C.c_long]),
    "pasc_gb300_vec_copy": (C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_void_p]),
    "pasc_gb300_vec_axpy": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_long, C.c_void_p]),
    "pasc_gb300_vec_waxpy": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_long, C.c_void_p]),
    "pasc_gb300_vec_scale": (C.c_int, [C.c_void_p, C.c_double, C.c_long, C.c_void_p]),
    "pasc_gb300_vec_dot": (C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.POINTER(C.c_double), C.c_void_p]),
    "pasc_gb300_permute_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_int, C.c_void_p]),
    "pasc_gb300_residual_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_long, C.c_int, C.c_double,
                                          C.c_void_p]),
    "pasc_gb300_theta_update_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_long, C.c_int, C.c_void_p]),
    "pasc_gb300_adjoint_default_opts": (None, [C.POINTER(AdjointOpts)]),
    "pasc_gb300_recon_mse": (C.c_int, [_h, _dp, C.POINTER(C.c_double)]),
    "pasc_gb300_polish_default_opts": (None, [C.POINTER(PolishOpts)]),
    "pasc_gb300_polish": (C.c_int, [_h, C.POINTER(PolishOpts), C.POINTER(PolishStats)]),
    "pasc_gb300_adjoint": (C.c_int, [_h, C.c_void_p, C.POINTER(AdjointOpts), C.POINTER(C.c_double), C.c_void_p,
                                     C.c_void_p, C.POINTER(AdjointStats)]),
    "pasc_gb300_batch_create": (C.c_int, [C.POINTER(_h), C.c_int, _lp, _ip, _dp, C.c_int]),
    "pasc_gb300_batch_destroy": (C.c_int, [_h]),
    "pasc_gb300_batch_size": (C.c_int, [_h, C.POINTER(C.c_int)]),
    "pasc_gb300_batch_set_loop": (C.c_int, [_h, C.c_int, C.c_int]),
    "pasc_gb300_batch_set_segment_tiles": (C.c_int, [_h, C.c_int]),
    "pasc_gb300_batch_get_segment_tiles": (C.c_int, [_h, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "pasc_gb300_batch_set_data": (C.c_int, [_h, C.c_int, _dp]),
    "pasc_gb300_batch_set_gamma": (C.c_int, [_h, C.c_int, _dp]),
    "pasc_gb300_batch_get_gamma": (C.c_int, [_h, C.c_int, _dp]),
    "pasc_gb300_batch_set_theta": (C.c_int, [_h, C.c_int, _dp]),
    "pasc_gb300_batch_get_theta": (C.c_int, [_h, C.c_int, _dp]),
    "pasc_gb300_batch_spgqp_solve": (C.c_int, [_h, C.POINTER(SpgqpOpts), C.c_void_p]),
    "pasc_gb300_batch_ts_solve": (C.c_int, [_h, C.POINTER(TsOpts), C.POINTER(SpgqpOpts), C.c_void_p]),
}

_lib = None


def lib_path() -> str:
    return LIB_PATH


def load(path: str | None = None):
    """Loads libpasc_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
                           " (the library has no CPU fallback)")
    L = C.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != PASC_OK:
        msg = load().pasc_gb300_last_error().decode(errors="replace")
        raise PascError(rc, msg)


def spgqp_opts(**kw) -> SpgqpOpts:
    o = SpgqpOpts()
    load().pasc_gb300_spgqp_default_opts(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


def ts_opts(**kw) -> TsOpts:
    o = TsOpts()
    load().pasc_gb300_ts_default_opts(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


def polish_opts(**kw) -> PolishOpts:
    o = PolishOpts()
    load().pasc_gb300_polish_default_opts(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


def adjoint_opts(**kw) -> AdjointOpts:
    o = AdjointOpts()
    load().pasc_gb300_adjoint_default_opts(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


class HostBuffer:
    """Page-locked host memory from pasc_gb300_host_alloc, freed when the object goes; `array`
    is a numpy view of it (keep the HostBuffer alive as long as the view is used)."""

    def __init__(self, n: int, dtype=np.float64):
        dt = np.dtype(dtype)
        ptr = C.c_void_p()
        check(load().pasc_gb300_host_alloc(C.byref(ptr), int(n) * dt.itemsize))
        self._ptr = ptr
        buf = (C.c_char * (int(n) * dt.itemsize)).from_address(ptr.value)
        self.array = np.frombuffer(buf, dtype=dt, count=int(n))

    def close(self):
        if getattr(self, "_ptr", None) is not None and self._ptr.value:
            self.array = None
            load().pasc_gb300_host_free(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def host_empty(n: int, dtype=np.float64) -> HostBuffer:
    """n values of page-locked host memory (see HostBuffer)."""
    return HostBuffer(n, dtype)
