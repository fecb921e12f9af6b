"""The C ABI library on a host without a GPU: it loads, exports every function declared in
include/pasc_gb300.h (and the ctypes binding declares each of them), reports the reference's
default settings, and fails cleanly (error code + message, no crash) when no device exists."""
import ctypes as C
import os
import re
import subprocess
import sys

import pytest

from pasc_inference_gb300 import build as B
from pasc_inference_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "pasc_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pasc_gb300_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    B.build()
    return capi.load()


def test_header_declares_functions():
    names = header_functions()
    assert "pasc_gb300_spgqp_solve" in names and "pasc_gb300_ts_solve" in names
    assert len(names) >= 25


def test_every_declared_symbol_is_exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", capi.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (pasc_gb300_\w+)", out))
    missing = [n for n in header_functions() if n not in exported]
    assert not missing, missing
    for n in header_functions():
        assert hasattr(lib, n)


def test_binding_covers_header():
    assert sorted(capi.PROTOTYPES) == header_functions()


def test_default_settings_are_the_references(lib):
    o = capi.spgqp_opts()
    # include/general/solver/spgqpsolver.h:19-36
    assert (o.maxit, o.eps, o.m, o.gamma, o.sigma1, o.sigma2, o.alphainit) == (1000, 1e-9, 20, 0.9, 0.0, 1.0, 2.0)
    assert (o.stop_difff, o.stop_normgp, o.stop_normgp_normb, o.stop_Anormgp, o.stop_Anormgp_normb) == (1, 0, 0, 0, 0)
    t = capi.ts_opts()
    # include/general/solver/tssolver.h:13-15
    assert (t.maxit, t.eps, t.init_permute, t.annealing, t.relative, t.thetasolved) == (300, 1e-6, 1, 1, 0, 0)
    assert lib.pasc_gb300_abi_version() == 1


def test_argument_errors_without_device(lib):
    h = C.c_void_p()
    assert lib.pasc_gb300_create(C.byref(h), 0, 3, 1, 1, 1.0, 0) == capi.PASC_ERR_ARG
    assert b"T must be" in lib.pasc_gb300_last_error()
    assert lib.pasc_gb300_create(C.byref(h), 100, 9, 1, 1, 1.0, 0) == capi.PASC_ERR_ARG
    assert lib.pasc_gb300_create(C.byref(h), 100, 3, 2, 0, 1.0, 0) == capi.PASC_ERR_NOTSUPP  # multichannel fp64
    assert lib.pasc_gb300_create(C.byref(h), 100, 3, 300, 1, 1.0, 0) == capi.PASC_ERR_NOTSUPP  # xdim > 256
    assert lib.pasc_gb300_create(C.byref(h), 100, 3, 0, 1, 1.0, 0) == capi.PASC_ERR_ARG
    assert lib.pasc_gb300_destroy(None) == capi.PASC_OK
    assert lib.pasc_gb300_spgqp_solve(None, None, None) == capi.PASC_ERR_ARG


def test_no_device_is_reported_not_crashed(lib):
    if lib.pasc_gb300_device_count() > 0:
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = lib.pasc_gb300_create(C.byref(h), 100, 3, 1, 1, 1.0, 0)
    assert rc == capi.PASC_ERR_CUDA
    assert b"no CUDA device" in lib.pasc_gb300_last_error()


NULL_SWEEP = r"""
import ctypes as C, sys
sys.path.insert(0, sys.argv[1])
from pasc_inference_gb300 import capi
L = C.CDLL(capi.LIB_PATH)
for name, (res, args) in capi.PROTOTYPES.items():
    creator = name in ("pasc_gb300_create", "pasc_gb300_create_graph", "pasc_gb300_batch_create")
    if not args or (args[0] is not capi._h and not creator):
        continue
    fn = getattr(L, name)
    fn.restype = C.c_int
    conv, vals = [], []
    for a in args:
        if a in (C.c_int, C.c_long, C.c_double, C.c_float):
            conv.append(a)
            vals.append(1 if creator else 0)
        else:
            conv.append(C.c_void_p)
            vals.append(None)
    fn.argtypes = conv
    print(name, fn(*vals), flush=True)
"""


def test_null_handles_and_pointers_are_refused(lib):
    """Every entry point that takes a handle or device pointer first, called with NULL for it
    and NULL / 0 for everything else, returns an error code (destroy, host_free, vec_free: OK) instead of crashing;
    the constructors refuse a NULL output pointer.  Run in a child process so that a crash
    fails this test and not the session."""
    r = subprocess.run([sys.executable, "-c", NULL_SWEEP, ROOT], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    rcs = dict(line.rsplit(" ", 1) for line in r.stdout.split("\n") if line.strip())
    assert len(rcs) >= 50, rcs
    for name, rc in rcs.items():
        if name in ("pasc_gb300_destroy", "pasc_gb300_batch_destroy", "pasc_gb300_host_free", "pasc_gb300_vec_free"):
            assert int(rc) == capi.PASC_OK, name
        else:
            assert int(rc) == capi.PASC_ERR_ARG, (name, rc)
