"""The projected Hermitian eigensolver (ncgm_heig) against numpy: the
shared-memory Jacobi (m <= 80, FP64 and double-float rotations) and the
multi-kernel tridiagonal solver (m > 80), on generic spectra and on
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
