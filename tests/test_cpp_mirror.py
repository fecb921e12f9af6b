"""The C++ class surface (include/pasc/pasc_gb300.hpp) over the C ABI: a driver written like the
reference's Signal1D example compiles against it, its host-side pieces (PETSc binary I/O, the
seeded gamma0 generator, errors as exceptions) behave as the Python package's, and on the GPU it
reaches exactly the result of the Python mirror on the same data file (same calls, same inputs,
deterministic kernels)."""
import os
import subprocess

import numpy as np
import pytest

from pasc_inference_gb300 import (Decomposition, GraphH1FEMModel, Signal1DData, TSSolver, capi,
                                  datagen, petscio)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pasc_inference_gb300")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not os.path.exists(capi.LIB_PATH):
        pytest.skip("libpasc_gb300.so not built")
    out = str(tmp_path_factory.mktemp("cpp") / "mirror_driver")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "mirror_driver.cpp"), "-L", PKG, "-lpasc_gb300",
                           "-Wl,-rpath," + PKG, "-o", out])
    return out


def test_host_side_pieces(driver, tmp_path):
    r = subprocess.run([driver, "--host-checks", str(tmp_path)], capture_output=True, text=True, check=True)
    lines = dict(l.split(" ", 1) for l in r.stdout.strip().splitlines())
    assert lines["roundtrip"] == "ok"
    u = np.array([float(v) for v in lines["uniform"].split()])
    assert np.array_equal(u, datagen.uniform(13, 0, 5))  # bit for bit
    assert lines["R=2"].split() == ["nodes", "2", "edges", "0", "grid", "17", "4"]
    assert np.allclose([float(v) for v in lines["scaled"].split()], [0.0, 1.0 / 3, 2.0 / 3, 1.0])
    assert np.allclose([float(v) for v in lines["unscaled"].split()], [-1.0, 0.0, 1.0, 2.0])
    assert int(lines["xdim=2"].split()[-1]) == capi.PASC_ERR_NOTSUPP
    assert int(lines["T=0"].split()[-1]) == capi.PASC_ERR_ARG
    # the file written by the C++ side is read back by the Python reader
    assert np.array_equal(petscio.load_vec(str(tmp_path / "roundtrip.bin")),
                          np.array([1.5, -2.25, 3.0e10, 0.0, -1e-300]))


@pytest.mark.gpu
def test_driver_matches_python_mirror(driver, tmp_path):
    sig = datagen.signal1d_cfg0()
    path = str(tmp_path / "signal.bin")
    petscio.save_vec(path, sig.data)
    r = subprocess.run([driver, path, "2", "10", str(tmp_path / "cpp")], capture_output=True, text=True, check=True)
    lines = dict(l.split(" ", 1) for l in r.stdout.strip().splitlines())
    L_cpp = float(lines["L"])
    th_cpp = np.array([float(v) for v in lines["theta"].split()])

    data = Signal1DData(path)
    data.set_decomposition(Decomposition(data.get_Tpreliminary(), 1, 2, 1, 1))
    model = GraphH1FEMModel(data, 10.0)
    model.problem.set_sweep_variant(1)  # as the driver does (the timed choice is per process)
    solver = TSSolver(data, options={"spgqpsolver_m": 10, "spgqpsolver_eps": 1e-6})
    solver.solve()
    assert L_cpp == solver.get_L()
    assert np.array_equal(th_cpp, data.get_thetavector())
    # saveSignal1D wrote the blocked gamma and the reconstruction
    g = petscio.load_vec(str(tmp_path / "cpp_gamma.bin"))
    rec = petscio.load_vec(str(tmp_path / "cpp_recovered.bin"))
    assert g.size == 2 * sig.T and rec.size == sig.T
    assert np.allclose(rec, g.reshape(2, -1).T @ th_cpp)


@pytest.mark.gpu
def test_image_driver_matches_python_mirror(driver, tmp_path):
    from pasc_inference_gb300 import BGMGraphGrid2D, ImageData
    w, h, K = 40, 30, 2
    rng = np.random.default_rng(4)
    yy, xx = np.mgrid[0:h, 0:w]
    truth = (((xx - w / 3) ** 2 + (yy - h / 2) ** 2) < (h / 4) ** 2).astype(float).ravel()
    img = truth + 0.4 * rng.standard_normal(w * h)
    path = str(tmp_path / "image.bin")
    petscio.save_vec(path, img)
    r = subprocess.run([driver, "--image", path, str(w), str(h), str(K), "2.0", str(tmp_path / "cpp")],
                       capture_output=True, text=True, check=True)
    lines = dict(l.split(" ", 1) for l in r.stdout.strip().splitlines())
    graph = BGMGraphGrid2D(w, h)
    graph.process_grid()
    data = ImageData(Decomposition(1, graph, K, 1, 1), path, w, h)
    GraphH1FEMModel(data, 2.0)
    solver = TSSolver(data, options={"spgqpsolver_m": 10, "spgqpsolver_eps": 1e-10})
    solver.solve()
    # one graph sweep kernel, same inputs: the two mirrors make the same calls
    assert float(lines["L"]) == solver.get_L()
    assert np.array_equal(np.array([float(v) for v in lines["theta"].split()]), data.get_thetavector())
    rec = petscio.load_vec(str(tmp_path / "cpp_recovered.bin"))
    g = petscio.load_vec(str(tmp_path / "cpp_gamma.bin"))
    assert rec.size == w * h and g.size == K * w * h
