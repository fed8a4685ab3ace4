"""GPU parity of the block GCG eigensolver (gcgm_complex_no_B_lock) against
the oracle's restatement, and convergence to exact eigenpairs."""
import numpy as np
import pytest

import nuclearcgm_gb300 as ng
from conftest import random_block, random_fields
from nuclearcgm_gb300 import abi, config
from oracle import oracle

pytestmark = pytest.mark.gpu


def _hams(n, a, seed, so=True, const_f=False):
    f, gradf, U, W, UC = random_fields(n, seed, so=so)
    if const_f:
        f = np.full(n ** 3, 20.7)
        gradf = np.zeros(3 * n ** 3)
    ctx = ng.Context(ng.Grid(n, a), 64)
    H = ng.Hamiltonian(ctx, abi.NEUTRON).set_fields(f, gradf, U, W)
    R = oracle.Hamiltonian.skyrme(n, a, f, gradf, U, W)
    return ctx, H, R


def _projector_gap(X, Y):
    """max |X X^H - Y Y^H| restricted to random probes (phase invariant)."""
    rng = np.random.default_rng(0)
    v = rng.normal(size=(X.shape[0], 3)) + 1j * rng.normal(size=(X.shape[0], 3))
    a = X @ (X.conj().T @ v)
    b = Y @ (Y.conj().T @ v)
    return np.abs(a - b).max() / np.abs(a).max()


def _orth(X):
    q, _ = np.linalg.qr(X)
    return np.asfortranarray(q)


def _phys(n, h):
    """Smooth physical-looking fields (mildly non-Hermitian H)."""
    from nuclearcgm_gb300 import workloads
    a, f, gradf, U, W = workloads.fields(n, h)
    ctx = ng.Context(ng.Grid(n, a), 64)
    H = ng.Hamiltonian(ctx, abi.NEUTRON).set_fields(f, gradf.T, U, W.T)
    R = oracle.Hamiltonian.skyrme(n, a, f, gradf.T, U, W.T)
    return ctx, H, R


@pytest.mark.parametrize("n,nev,pcols", [(10, 8, 0), (12, 6, 6), (9, 5, 3)])
def test_one_gcg_step_fixed_pcg_length_matches_oracle(n, nev, pcols):
    """One outer iteration with all 80 PCG steps taken (cgTol = 0), so both
    sides apply the same operator sequence: Ritz values agree to rounding."""
    ctx, H, R = _phys(n, 0.9)
    N = 2 * n ** 3
    X0 = random_block(N, nev, 1)
    P = None
    if pcols:
        P = random_block(N, pcols, 2)
        P /= np.linalg.norm(P, axis=0)
    prm = abi.GcgParams(max_iter=1, tol=1e-6, cg_steps=80, cg_tol=0.0,
                        shift=0.0, ordering=abi.ORDER_ASCENDING,
                        precision=abi.FP64, precond=0)
    Xg, lg, st = H.gcg(X0, nev, P, prm)
    Xo, lo, info = R.gcg(X0, nev, P, 0.0, 1, 1e-6, 80, 0.0, 1)
    assert np.allclose(lg, lo, rtol=1e-8, atol=1e-8)
    assert _projector_gap(Xg, Xo) < 1e-7
    assert st.basis_cols == info["basis_cols"]


def test_wide_search_space_matches_oracle():
    """nev = 32 with 32 conjugate directions: a 96-column search space, past
    the shared-memory tier, so the multi-kernel Cholesky-with-drop and
    eigensolver run (FP64 form). With 32 unconverged columns the 80-step PCG
    amplifies rounding differences between the two machines to ~1e-8 of the
    Ritz values (measured at nev = 32 without directions, where the
    small-tier kernels run, too), hence the looser bounds of this case."""
    precision = abi.FP64
    n, nev, pcols = 10, 32, 32
    ctx, H, R = _phys(n, 0.9)
    N = 2 * n ** 3
    X0 = random_block(N, nev, 1)
    P = random_block(N, pcols, 2)
    P /= np.linalg.norm(P, axis=0)
    prm = abi.GcgParams(max_iter=1, tol=1e-6, cg_steps=80, cg_tol=0.0,
                        shift=0.0, ordering=abi.ORDER_ASCENDING,
                        precision=precision, precond=0)
    Xg, lg, st = H.gcg(X0, nev, P, prm)
    Xo, lo, info = R.gcg(X0, nev, P, 0.0, 1, 1e-6, 80, 0.0, 1)
    print("wide search space: %d columns, max |dlambda| %.2e MeV, projector "
          "gap %.2e" % (st.basis_cols, np.abs(lg - lo).max(),
                        _projector_gap(Xg, Xo)))
    assert st.basis_cols > 80
    assert np.allclose(lg, lo, rtol=1e-7)
    assert _projector_gap(Xg, Xo) < 1e-4


def test_wide_search_space_tensor_core_step_is_consistent():
    """The tensor-core form on the same 96-column search space. From a random
    block its single step follows another PCG trajectory than FP64 (FP32
    corrections of an indefinite shifted system; both are upper bounds of the
    true levels), so the check is self-consistency: the returned block is
    orthonormal and each Ritz value equals the Rayleigh quotient of its vector
    under the oracle's CSR Hamiltonian. The Hamiltonian is made Hermitian
    (constant f, no spin-orbit field) so that the Rayleigh quotient is the
    quantity the lower-triangle Rayleigh-Ritz step returns."""
    n, nev, pcols = 10, 32, 32
    ctx, H, R = _hams(n, 0.5 * (n - 1) * 0.9, 77, so=False, const_f=True)
    N = 2 * n ** 3
    X0 = random_block(N, nev, 1)
    P = random_block(N, pcols, 2)
    P /= np.linalg.norm(P, axis=0)
    prm = abi.GcgParams(max_iter=1, tol=1e-6, cg_steps=80, cg_tol=0.0,
                        shift=0.0, ordering=abi.ORDER_ASCENDING,
                        precision=abi.FP32_TC, precond=0)
    Xg, lg, st = H.gcg(X0, nev, P, prm)
    assert st.basis_cols > 80
    orth = np.abs(Xg.conj().T @ Xg - np.eye(nev)).max()
    rq = np.real(np.einsum("ij,ij->j", Xg.conj(), R.apply(Xg)))
    print("tensor-core wide step: orthonormality %.1e, max |RQ - lambda| "
          "%.1e MeV" % (orth, np.abs(rq - lg).max()))
    assert orth < 1e-10
    assert np.abs(rq - lg).max() < 1e-6 * np.abs(lg).max()


@pytest.mark.parametrize("n,nev,pcols", [(10, 8, 0), (12, 6, 6), (9, 5, 3)])
def test_one_hf_gcg_step_matches_oracle(n, nev, pcols):
    """One outer iteration with the HF parameters (1, 1e-6, 80, 1e-5): the
    PCG stopping test may fall on either side of the threshold on the two
    machines, so the Ritz values agree to the correction's accuracy."""
    a = 0.5 * (n - 1) * 0.8
    ctx, H, R = _hams(n, a, 40 + n)
    N = 2 * n ** 3
    X0 = random_block(N, nev, 1)
    P = None
    if pcols:
        P = random_block(N, pcols, 2)
        P /= np.linalg.norm(P, axis=0)
    prm = config._gcg(config.HF_GCG)
    Xg, lg, st = H.gcg(X0, nev, P, prm)
    Xo, lo, info = R.gcg(X0, nev, P, 0.0, 1, 1e-6, 80, 1e-5, 1)
    assert np.allclose(lg, lo, rtol=1e-6)
    assert st.basis_cols == info["basis_cols"]
    assert st.iterations == 1


def test_converges_to_exact_lowest_eigenpairs():
    import scipy.sparse as sp
    n, a, nev = 8, 5.0, 6
    ctx, H, R = _hams(n, a, 3, so=False, const_f=True)
    N = 2 * n ** 3
    rp, col, val = R.csr()
    dense = sp.csr_matrix((val, col, rp), shape=(N, N)).toarray()
    ref = np.linalg.eigvalsh(dense)[:nev]
    X0 = random_block(N, nev, 4)
    prm = abi.GcgParams(max_iter=60, tol=1e-9, cg_steps=40, cg_tol=1e-9,
                        shift=0.0, ordering=abi.ORDER_ASCENDING,
                        precision=abi.FP64, precond=0)
    X, lam, st = H.gcg(X0, nev, None, prm)
    assert np.allclose(lam, ref, atol=1e-8)
    HX = R.apply(X)
    assert np.abs(HX - X * lam).max() < 1e-6


def test_fp32_correction_reaches_same_eigenvalues():
    """Mixed form: PCG in FP32, Rayleigh-Ritz and residuals in FP64."""
    n, nev = 10, 8
    ctx, H, R = _phys(n, 0.9)
    N = 2 * n ** 3
    X0 = random_block(N, nev, 6)
    p64 = abi.GcgParams(max_iter=40, tol=1e-8, cg_steps=40, cg_tol=1e-6,
                        shift=0.0, ordering=abi.ORDER_ASCENDING,
                        precision=abi.FP64, precond=0)
    p32 = abi.GcgParams(max_iter=40, tol=1e-8, cg_steps=40, cg_tol=1e-6,
                        shift=0.0, ordering=abi.ORDER_ASCENDING,
                        precision=abi.FP32, precond=0)
    _, l64, _ = H.gcg(X0, nev, None, p64)
    X32, l32, _ = H.gcg(X0, nev, None, p32)
    # row-point fields make H non-Hermitian: the Ritz values of the
    # lower-triangle projection converge, the residual AX - X L does not
    # vanish; compare the converged Ritz values (and the oracle's)
    _, lo, _ = R.gcg(X0, nev, None, 0.0, 40, 1e-8, 40, 1e-6, 1)
    # the two highest Ritz values of the block converge slowest; compare the
    # converged ones
    k = nev - 2
    assert np.allclose(l32[:k], l64[:k], rtol=1e-8, atol=1e-8)
    assert np.allclose(l64[:k], lo[:k], rtol=1e-8, atol=1e-8)


def test_rank_deficient_block_drops_columns():
    """Duplicated columns are dropped like modified Gram-Schmidt does."""
    n, a, nev = 8, 4.0, 4
    ctx, H, R = _hams(n, a, 9)
    N = 2 * n ** 3
    X0 = random_block(N, nev, 7)
    X0[:, 3] = X0[:, 1]  # dependent column
    prm = config._gcg(config.HF_GCG)
    Xg, lg, st = H.gcg(X0, nev, None, prm)
    Xo, lo, info = R.gcg(X0, nev, None, 0.0, 1, 1e-6, 80, 1e-5, 1)
    assert np.all(np.isfinite(lg))
    assert st.basis_cols == info["basis_cols"]
    assert np.allclose(lg, lo, rtol=1e-8, atol=1e-8)
