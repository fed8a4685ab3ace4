"""The header-only C++ shim (include/ncgm_reference.hpp) compiles and links
against libncgm.so like the reference's run loop would; on a GPU it solves a
known-answer Hamiltonian (harmonic oscillator levels hbar w (N + 3/2))."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    from nuclearcgm_gb300 import build
    build.build()
    exe = str(tmp_path / "shim_smoke")
    lib = os.path.join(ROOT, "nuclearcgm_gb300")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "shim_smoke.cpp"), "-L", lib,
           "-lncgm", "-Wl,-rpath," + lib, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def test_shim_compiles_links_and_reports_no_device(tmp_path):
    import torch
    exe = _build(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is visible")
    out = subprocess.run([exe], capture_output=True, text=True, check=True)
    assert out.stdout.startswith("no-device")


@pytest.mark.gpu
def test_shim_solves_harmonic_oscillator(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, check=True)
    lam = np.array([float(x) for x in out.stdout.split()])
    assert np.allclose(lam[:2], 15.0, rtol=5e-3)
    assert np.allclose(lam[2:8], 25.0, rtol=5e-3)


def _build_eigen(tmp_path):
    from nuclearcgm_gb300 import build
    build.build()
    exe = str(tmp_path / "shim_eigen")
    lib = os.path.join(ROOT, "nuclearcgm_gb300")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror",
           "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "tests", "cpp", "eigen_stub"),
           os.path.join(ROOT, "tests", "cpp", "shim_eigen.cpp"), "-L", lib,
           "-lncgm", "-Wl,-rpath," + lib, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def test_eigen_overloads_and_edf_compile_and_run(tmp_path):
    """The NCGM_WITH_EIGEN overloads (MatrixXcd in and out, as the
    reference's run loop passes them) compile against a declaration-level
    Eigen stand-in, and EDF(functional) on a functional-file object gives
    the coupling constants of EDF::setFromInteraction (include/EDF.hpp:
    25-31, src/skyrme/EDF.cpp:4-59)."""
    import torch
    from nuclearcgm_gb300 import config
    exe = _build_eigen(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is visible")
    out = subprocess.run([exe], capture_output=True, text=True,
                         check=True).stdout.split("\n")
    e = config.edf_from_skyrme(config.FUNCTIONALS["SLy4"])
    words = out[0].split()
    assert words[0] == "edf"
    assert float(words[1]) == pytest.approx(e.C0rr, abs=1e-9)
    assert float(words[2]) == pytest.approx(e.C1rr, abs=1e-9)
    assert float(words[3]) == pytest.approx(e.C0nJ, abs=1e-9)
    assert float(words[4]) == pytest.approx(e.C1nJ, abs=1e-9)
    assert out[1] == "no-device"


@pytest.mark.gpu
def test_eigen_overloads_solve_on_device(tmp_path):
    exe = _build_eigen(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True,
                         check=True).stdout.split("\n")
    words = out[1].split()
    assert words[0] == "solved" and words[1] == "8" and words[2] == "8"
    # the harmonic-oscillator ground level 3/2 hbar w = 15 MeV
    assert float(words[3]) == pytest.approx(15.0, rel=5e-3)
    assert words[4] == "8"
