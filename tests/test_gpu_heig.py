"""The projected Hermitian eigensolver (ncgm_heig) against numpy: the
shared-memory FP64 Jacobi (FP64 form, m <= 80), the one-CTA double-float
Householder method (FP32 forms, m <= 112), the double-float Jacobi
(NCGM_HEIG_MID=0, m <= 80, in a child process) and the multi-kernel
tridiagonal solver (above those sizes), on generic spectra and on
time-reversal symmetric matrices whose levels are all twofold (Kramers)."""
import numpy as np
import pytest

import nuclearcgm_gb300 as ng
from nuclearcgm_gb300 import abi

pytestmark = pytest.mark.gpu


def _herm(m, rng, kramers):
    if kramers:
        h = m // 2
        B = rng.normal(size=(h, h)) + 1j * rng.normal(size=(h, h))
        B = B + B.conj().T
        C = rng.normal(size=(h, h)) + 1j * rng.normal(size=(h, h))
        C = C - C.T
        return np.block([[B, C], [-C.conj(), B.conj()]])
    B = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
    return B + B.conj().T + np.diag(np.linspace(-30, 30, m))


@pytest.mark.parametrize("m,kramers,precision", [
    (24, False, abi.FP64), (60, True, abi.FP32), (80, False, abi.FP32_TC),
    (2, False, abi.FP32), (24, True, abi.FP32), (48, False, abi.FP32_TC),
    (100, True, abi.FP32), (112, False, abi.FP32_TC), (114, True, abi.FP32),
    (81, False, abi.FP64), (150, True, abi.FP64), (192, False, abi.FP32),
    (320, True, abi.FP64), (480, False, abi.FP64)])
def test_heig_matches_numpy(m, kramers, precision):
    rng = np.random.default_rng(m + 7 * kramers)
    A = np.asfortranarray(_herm(m, rng, kramers))
    m = A.shape[0]
    ctx = ng.Context(ng.Grid(8, 3.0), 2)
    w = np.zeros(m)
    V = np.zeros((m, m), np.complex128, order="F")
    ng._check(ng.load().ncgm_heig(ctx.h, A.ctypes.data, m, w.ctypes.data,
                                  V.ctypes.data, precision))
    ref = np.linalg.eigvalsh(A)
    scale = np.abs(ref).max()
    eig = np.abs(w - ref).max() / scale
    orth = np.abs(V.conj().T @ V - np.eye(m)).max()
    res = np.abs(A @ V - V * w).max() / scale
    print("m=%d kramers=%s: eigenvalues %.1e, orthonormality %.1e, "
          "residual %.1e" % (m, kramers, eig, orth, res))
    assert eig <= 1e-12 and orth <= 1e-10 and res <= 1e-11
    ctx.close()


_MID_CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import nuclearcgm_gb300 as ng
from test_gpu_heig import _herm
m, kramers, prec = int(sys.argv[2]), sys.argv[3] == "1", int(sys.argv[4])
A = np.asfortranarray(_herm(m, np.random.default_rng(m + 7 * kramers), kramers))
m = A.shape[0]
ctx = ng.Context(ng.Grid(8, 3.0), 2)
w = np.zeros(m)
V = np.zeros((m, m), np.complex128, order="F")
ng._check(ng.load().ncgm_heig(ctx.h, A.ctypes.data, m, w.ctypes.data,
                              V.ctypes.data, prec))
ref = np.linalg.eigvalsh(A)
scale = np.abs(ref).max()
print(np.abs(w - ref).max() / scale, np.abs(V.conj().T @ V - np.eye(m)).max(),
      np.abs(A @ V - V * w).max() / scale)
"""


@pytest.mark.parametrize("m,kramers", [(2, False), (24, True), (60, True),
                                       (80, False)])
def test_heig_double_float_jacobi(m, kramers):
    """The double-float Jacobi that the FP32 forms used before the one-CTA
    Householder method (NCGM_HEIG_MID=0 selects it; the switch is read once
    per process, so a child runs it)."""
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    env = dict(os.environ, NCGM_HEIG_MID="0")
    out = subprocess.run([sys.executable, "-c", _MID_CHILD,
                          os.path.dirname(here), str(m), str(int(kramers)),
                          str(abi.FP32)], env=env, capture_output=True,
                         text=True, cwd=here, check=True).stdout.split()
    eig, orth, res = (float(x) for x in out)
    print("double-float Jacobi m=%d kramers=%s: eigenvalues %.1e, "
          "orthonormality %.1e, residual %.1e" % (m, kramers, eig, orth, res))
    assert eig <= 1e-12 and orth <= 1e-10 and res <= 1e-11
