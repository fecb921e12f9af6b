"""The GB300 backend of the reference's generic solvers (include/pasc/gb300_backend.hpp) compiles
and links against the reference's unmodified generic headers: the driver translation unit that
oracle/build_ref.sh writes (the reference's headers inlined) is compiled with g++ and linked to
libpasc_gb300.so.  No GPU is needed for this; tests/test_gpu_backend.py runs it."""
import os
import subprocess

import pytest

from pasc_inference_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FLAT = os.path.join(ROOT, "oracle", "_ref", "backend", "gb300_backend_driver_flat.cpp")


def test_backend_driver_compiles_and_links(tmp_path):
    from oracle import pasc_oracle as O
    O.build_ref()
    if not os.path.exists(FLAT):
        pytest.skip("oracle/build_ref.sh found no reference tree")
    B.build()
    exe = tmp_path / "driver"
    r = subprocess.run(["g++", "-std=c++14", "-O2", "-w", "-I", os.path.join(ROOT, "include"), FLAT, "-L", B.PKG,
                        "-lpasc_gb300", "-Wl,-rpath," + B.PKG, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # the driver runs (no GPU needed to start it) and refuses an empty input file
    fin = tmp_path / "in.bin"
    fin.write_bytes(b"")
    r = subprocess.run([str(exe), str(fin), str(tmp_path / "out.bin")], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0
