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
