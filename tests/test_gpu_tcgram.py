"""Tensor-core Gram products (tcgen05 kind::tf32, split TF32 operands) of
the mixed-precision GCG against the FP64 Gram and numpy."""
import numpy as np
import pytest

import nuclearcgm_gb300 as ng
from nuclearcgm_gb300 import abi, workloads

pytestmark = pytest.mark.gpu


def _gram(ctx, A, B, precision):
    import ctypes as C
    A = np.asfortranarray(A, np.complex128)
    B = np.asfortranarray(B, np.complex128)
    Cm = np.zeros((A.shape[1], B.shape[1]), np.complex128, order="F")
    ng._check(ng.load().ncgm_gram(ctx.h, A.ctypes.data, A.shape[1],
                                  B.ctypes.data, B.shape[1], Cm.ctypes.data,
                                  precision))
    return Cm


@pytest.mark.parametrize("n,p,q", [(12, 5, 7), (16, 24, 24), (30, 32, 32),
                                   (20, 70, 40), (24, 3, 100)])
def test_tensor_core_gram(n, p, q):
    N = 2 * n ** 3
    ctx = ng.Context(ng.Grid(n, 0.5 * (n - 1) * 0.6), 4)
    rng = np.random.default_rng(n + p + q)
    A = workloads.orthonormal_block(N, p, seed=n + p)
    B = (rng.normal(size=(N, q)) + 1j * rng.normal(size=(N, q))) * 0.01
    ref = A.conj().T @ B
    g64 = _gram(ctx, A, B, abi.FP64)
    g32 = _gram(ctx, A, B, abi.FP32)
    scale = np.abs(ref).max()
    assert np.abs(g64 - ref).max() <= 1e-13 * scale
    err = np.abs(g32 - ref).max() / scale
    print("n=%d p=%d q=%d: tensor-core Gram max error %.2e (relative)" % (
        n, p, q, err))
    assert err <= 2e-5
    ctx.close()


def test_tensor_core_gram_orthonormal_block():
    """A^H A of an orthonormal block: the identity to FP32-level error."""
    n, p = 24, 48
    ctx = ng.Context(ng.Grid(n, 7.0), 4)
    A = workloads.orthonormal_block(2 * n ** 3, p, seed=5)
    g = _gram(ctx, A, A, abi.FP32)
    assert np.abs(g - np.eye(p)).max() <= 2e-5
    ctx.close()


@pytest.mark.parametrize("n,p,q", [(12, 5, 7), (16, 24, 24), (30, 32, 32),
                                   (20, 70, 40), (24, 3, 100)])
def test_exact_digit_gram(n, p, q):
    """The exact-digit tensor-core form (NCGM_FP32_TC): FP64-level error."""
    N = 2 * n ** 3
    ctx = ng.Context(ng.Grid(n, 0.5 * (n - 1) * 0.6), 4)
    rng = np.random.default_rng(7 * n + p + q)
    A = workloads.orthonormal_block(N, p, seed=n + 2 * p)
    B = (rng.normal(size=(N, q)) + 1j * rng.normal(size=(N, q))) * 0.01
    B[:, 0] *= 1e-6  # a column far below the others: per-column scaling
    ref = A.conj().T @ B
    g = _gram(ctx, A, B, abi.FP32_TC)
    err = np.abs(g - ref).max() / np.abs(ref).max()
    col0 = np.abs(g[:, 0] - ref[:, 0]).max() / np.abs(ref[:, 0]).max()
    print("n=%d p=%d q=%d: exact-digit Gram max error %.2e (column 0: %.2e)"
          % (n, p, q, err, col0))
    assert err <= 5e-12 and col0 <= 5e-12
    ctx.close()


@pytest.mark.parametrize("n,p", [(12, 5), (16, 70), (30, 32), (24, 100)])
def test_exact_digit_self_gram(n, p):
    """A^H A with both operands the same buffer: the block is digitised once
    and output tiles inside its own digit tile read B from there."""
    N = 2 * n ** 3
    ctx = ng.Context(ng.Grid(n, 0.5 * (n - 1) * 0.6), 4)
    A = workloads.orthonormal_block(N, p, seed=3 * n + p)
    A[:, 0] *= 1e-6
    A[:, -1] *= 3.0
    ref = A.conj().T @ A
    g = _gram(ctx, A, A, abi.FP32_TC)
    # the digit error of entry (i, j) scales with |a_i| |a_j| (per-column
    # scaling), so it is measured against sqrt(G_ii G_jj)
    d = np.sqrt(np.abs(np.diag(ref)))
    err = (np.abs(g - ref) / np.outer(d, d)).max()
    print("n=%d p=%d: exact-digit self Gram max error %.2e (of |a_i| |a_j|)"
          % (n, p, err))
    assert err <= 5e-12
    assert (np.abs(g - g.conj().T) / np.outer(d, d)).max() <= 5e-12
    ctx.close()


def _vc(ctx, V, Cm, precision):
    V = np.asfortranarray(V, np.complex128)
    Cm = np.asfortranarray(Cm, np.complex128)
    Y = np.zeros((V.shape[0], Cm.shape[1]), np.complex128, order="F")
    ng._check(ng.load().ncgm_vc(ctx.h, V.ctypes.data, V.shape[1],
                                Cm.ctypes.data, Cm.shape[1], Y.ctypes.data,
                                precision))
    return Y


@pytest.mark.parametrize("n,m,k", [(12, 5, 7), (16, 24, 24), (20, 70, 40),
                                   (24, 3, 100), (16, 192, 64), (10, 33, 1)])
def test_exact_digit_subspace_rotation(n, m, k):
    """Y = V C on the tensor cores (exact digit products) against the FP64
    kernel and numpy: ~1e-12 relative, also for a column of V far below the
    others and for ragged tiles (m, k not multiples of the tile sizes)."""
    N = 2 * n ** 3
    ctx = ng.Context(ng.Grid(n, 0.5 * (n - 1) * 0.6), 4)
    rng = np.random.default_rng(11 * n + m + k)
    V = workloads.orthonormal_block(N, m, seed=n + 3 * m)
    V[:, 0] *= 1e-6
    Cm = rng.normal(size=(m, k)) + 1j * rng.normal(size=(m, k))
    ref = V @ Cm
    y64 = _vc(ctx, V, Cm, abi.FP64)
    ytc = _vc(ctx, V, Cm, abi.FP32_TC)
    scale = np.abs(ref).max()
    assert np.abs(y64 - ref).max() <= 1e-13 * scale
    err = np.abs(ytc - ref).max() / scale
    print("n=%d m=%d k=%d: exact-digit V C max error %.2e (relative)" % (
        n, m, k, err))
    assert err <= 5e-12
    ctx.close()
