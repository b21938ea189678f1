"""The C++ drop-in header include/ssim_gb.hpp: ssim::fem::basic_time_step's method names over the C ABI.

tests/cpp/drop_in.cpp is a host program written against the header.  Without a GPU it checks the host-only
utilities, that construction fails with ssim::gb300::cuda_error and that an invalid argument maps to
std::invalid_argument (time_step.hpp:316-374).  On a GPU it steps a scene with Newton through the C++
class, and the state must equal, bitwise, the same steps through the Python binding of the same library.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    from ssim_gb300 import _lib

    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libssim_gb300.so is not built")
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "drop_in")
    lib_dir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "drop_in.cpp"), "-o", exe, "-L", lib_dir, "-lssim_gb300",
                    f"-Wl,-rpath,{lib_dir}"], check=True, capture_output=True, text=True)
    return exe


def test_cpp_header_cpu_error_path(tmp_path):
    import torch

    if torch.cuda.is_available():
        pytest.skip("checks the no-GPU error path")
    r = subprocess.run([_build(tmp_path), "cpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "cpu ok" in r.stdout


@pytest.mark.gpu
def test_cpp_header_steps_like_python_binding(tmp_path):
    import ssim_gb300 as g
    from ssim_gb300 import mesh

    X, T = mesh.kuhn_box((6, 4, 4), (1.5, 1.0, 1.0))
    fixed = np.where(X[:, 0] == 0.0)[0].astype(np.int32)
    scene = tmp_path / "scene.bin"
    with open(scene, "wb") as f:
        f.write(np.array([X.shape[0], T.shape[0], fixed.size], dtype=np.int32).tobytes())
        f.write(np.ascontiguousarray(X, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(T, dtype=np.int32).tobytes())
        f.write(fixed.tobytes())
    out = tmp_path / "u.bin"
    r = subprocess.run([_build(tmp_path), "gpu", str(scene), str(out), "3"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    u_cpp = np.fromfile(out, dtype=np.float64).reshape(-1, 3)

    ts = g.TimeStep(X, T, 1e-2, 1e5, 0.45, 1000.0)
    ts.mark_dirichlet_batched(fixed, np.zeros((fixed.size, 3)))
    ts.add_gravity([0.0, 0.0, -9.8])
    ts.set_params(g.default_params(stop_mode=1, rel_tol=1e-10, cg_rtol=1e-12))
    ts.reset("newton")
    for _ in range(3):
        ts.prepare_step()
        ts.compute_step()
        ts.step_next()
        assert ts.stats()["converged"] == 1
    assert np.array_equal(u_cpp, ts.get("deformation"))
    assert u_cpp[:, 2].min() < 0
