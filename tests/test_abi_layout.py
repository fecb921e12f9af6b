"""The ctypes binding against include/pasc_gb300.h itself, on the CPU: every struct of the header
has the size and field offsets its ctypes Structure gives (measured by a C program compiled from
the header with gcc), and every function's return and argument types agree with its ctypes
prototype, argument by argument.  A mismatch in either would pass name checks and corrupt
memory at the first call."""
import ctypes as C
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from pasc_inference_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pasc_gb300.h")

# header struct -> ctypes Structure of the binding
STRUCTS = {
    "pasc_gb300_spgqp_opts": capi.SpgqpOpts,
    "pasc_gb300_spgqp_stats": capi.SpgqpStats,
    "pasc_gb300_ts_opts": capi.TsOpts,
    "pasc_gb300_ts_stats": capi.TsStats,
    "pasc_gb300_adjoint_opts": capi.AdjointOpts,
    "pasc_gb300_adjoint_stats": capi.AdjointStats,
    "pasc_gb300_polish_opts": capi.PolishOpts,
    "pasc_gb300_polish_stats": capi.PolishStats,
}
HANDLES = ("pasc_gb300_problem", "pasc_gb300_batch")

SCALARS = {"int": C.c_int, "long": C.c_long, "unsigned long": C.c_ulong, "double": C.c_double,
           "float": C.c_float}
# the binding's array arguments (numpy arrays of that dtype)
ARRAYS = {"double": capi._dp, "float": capi._fp, "int": capi._ip, "long": capi._lp}


def _source():
    src = open(HEADER).read()
    return re.sub(r"/\*.*?\*/", " ", src, flags=re.S)


def header_structs():
    """name -> [field, ...] of every `typedef struct { ... } name;`"""
    out = {}
    for body, name in re.findall(r"typedef\s+struct\s*\{(.*?)\}\s*(\w+)\s*;", _source(), flags=re.S):
        out[name] = [re.findall(r"(\w+)\s*(?:\[[^\]]*\])?\s*$", d.strip())[0] for d in body.split(";") if d.strip()]
    return out


def _parse_type(decl: str):
    """('base type', pointer depth) of a parameter or return declaration without its name."""
    depth = decl.count("*")
    base = " ".join(t for t in decl.replace("*", " ").split() if t != "const")
    return base, depth


def header_prototypes():
    """name -> (return type, [parameter types]) of every function of the header."""
    out = {}
    for ret, name, params in re.findall(r"([\w\s\*]+?)\b(pasc_gb300_\w+)\s*\(([^;{]*?)\)\s*;", _source()):
        ret = ret.split("\n")[-1].strip()
        plist = []
        params = " ".join(params.split())
        if params not in ("", "void"):
            for p in params.split(","):
                p = p.strip()
                m = re.match(r"(.*?[\s\*])(\w+)$", p)
                assert m, (name, p)
                plist.append(_parse_type(m.group(1)))
        out[name] = (_parse_type(ret), plist)
    return out


def test_header_parses():
    structs, protos = header_structs(), header_prototypes()
    assert set(structs) == set(STRUCTS), sorted(structs)
    assert sorted(protos) == sorted(capi.PROTOTYPES)
    assert protos["pasc_gb300_spgqp_solve"] == (("int", 0), [("pasc_gb300_problem", 1),
                                                              ("pasc_gb300_spgqp_opts", 1),
                                                              ("pasc_gb300_spgqp_stats", 1)])


def test_struct_layouts_match_ctypes(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    structs = header_structs()
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void) {"]
    for name, fields in structs.items():
        lines.append(f'printf("{name} sizeof %zu\\n", sizeof({name}));')
        for f in fields:
            lines.append(f'printf("{name} {f} %zu\\n", offsetof({name}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", str(src), "-o", str(exe)], check=True)
    measured = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        s, f, v = line.split()
        measured[(s, f)] = int(v)
    for name, cls in STRUCTS.items():
        assert [f for f, _ in cls._fields_] == structs[name], name
        assert C.sizeof(cls) == measured[(name, "sizeof")], name
        for f, _ in cls._fields_:
            assert getattr(cls, f).offset == measured[(name, f)], (name, f)


def _expected_ok(ctype, decl):
    """Whether the binding's ctypes type can carry the header's declared type."""
    base, depth = decl
    if depth == 0:
        return ctype is SCALARS.get(base)
    if base in HANDLES:
        return ctype is capi._h if depth == 1 else ctype == C.POINTER(capi._h)
    if depth == 1 and base in STRUCTS:
        # one struct, or an array of them (the batch's per-signal results) by address
        return ctype == C.POINTER(STRUCTS[base]) or ctype is C.c_void_p
    if depth == 1 and base == "void":
        return ctype is C.c_void_p
    if depth == 2 and (base == "void" or base in SCALARS):
        # an output address (vec_alloc's device pointer): a pointer to a pointer-sized slot
        return ctype == C.POINTER(C.c_void_p)
    if depth == 1 and base in SCALARS:
        # device arrays travel as addresses; host arrays as numpy arrays of the same dtype;
        # single results as pointers to the scalar
        return ctype is C.c_void_p or ctype is ARRAYS.get(base) or ctype == C.POINTER(SCALARS[base])
    return False


def test_prototypes_match_ctypes():
    protos = header_prototypes()
    bad = []
    for name, (res, args) in capi.PROTOTYPES.items():
        ret, params = protos[name]
        if ret == ("void", 0):
            ok_ret = res is None
        elif ret == ("char", 1):
            ok_ret = res is C.c_char_p
        else:
            ok_ret = _expected_ok(res, ret)
        if not ok_ret:
            bad.append((name, "return", ret, res))
        if len(args) != len(params):
            bad.append((name, "arity", len(params), len(args)))
            continue
        for i, (a, p) in enumerate(zip(args, params)):
            if not _expected_ok(a, p):
                bad.append((name, i, p, a))
    assert not bad, bad


def test_long_arrays_use_the_c_long_width():
    assert np.dtype(capi.LONG_DTYPE).itemsize == C.sizeof(C.c_long)


def test_checker_rejects_wrong_types():
    """The rules above refuse what would corrupt a call: a long for an int, an array of the wrong
    dtype, another struct."""
    assert not _expected_ok(C.c_long, ("int", 0))
    assert not _expected_ok(capi._fp, ("double", 1))
    assert not _expected_ok(C.POINTER(capi.TsOpts), ("pasc_gb300_spgqp_opts", 1))
    assert not _expected_ok(C.c_double, ("float", 0))
