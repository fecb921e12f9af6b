"""Builds the GB300 library in-tree: pasc_inference_gb300/libpasc_gb300.so.

Every .cu translation unit under pasc_inference_gb300/csrc is compiled for sm_103a only
(`-gencode arch=compute_103a,code=sm_103a`), in parallel, then linked with nvcc into one
shared library exporting the C ABI of include/pasc_gb300.h.  nvcc cross-compiles, so this
runs on a machine without a GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(PKG, "_build")
LIB_NAME = "libpasc_gb300.so"
LIB_PATH = os.path.join(PKG, LIB_NAME)

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_flags: list[str] | None = None) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    srcs = sources()
    objs = []
    jobs = []
    flags = NVCC_FLAGS + (extra_flags or [])
    for s in srcs:
        o = os.path.join(BUILD_DIR, os.path.splitext(os.path.basename(s))[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc(), *ARCH_FLAGS, *flags, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if verbose or r.returncode != 0:
                    sys.stderr.write(" ".join(j) + "\n" + r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed for {j[-3]}")
    if force or jobs or _stale(LIB_PATH, objs):
        cmd = [nvcc(), *ARCH_FLAGS, "-shared", "-o", LIB_PATH, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link of libpasc_gb300.so failed")
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
