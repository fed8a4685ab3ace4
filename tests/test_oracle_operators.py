"""CPU checks that pin the FP64 oracle: analytic derivatives, trapezoid
integral, the assembled Hamiltonian against an independent numpy restatement
of the term formulas, and Hermitian structure."""
import numpy as np
import pytest

from conftest import random_block, random_fields
from oracle import oracle


def _xyz(n, a):
    h = 2 * a / (n - 1)
    xs = -a + np.arange(n) * h
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    return X.ravel(), Y.ravel(), Z.ravel(), h


def test_integral_constant_and_quadratic():
    n, a = 14, 6.5
    assert oracle.integral(n, a, np.ones(n ** 3)) == pytest.approx((2 * a) ** 3,
                                                                   rel=1e-13)
    x, y, z, h = _xyz(n, a)
    # trapezoid rule on x^2 over [-a, a]: exact value of the composite rule
    xs = -a + np.arange(n) * h
    w = np.full(n, h)
    w[0] = w[-1] = h / 2
    tz = (w * xs ** 2).sum() * (2 * a) ** 2
    assert oracle.integral(n, a, x ** 2) == pytest.approx(tz, rel=1e-13)


def test_gradient_exact_on_linear_and_cubic():
    n, a = 16, 7.5
    x, y, z, h = _xyz(n, a)
    g = oracle.grad_nospin(n, a, 2 * x - 3 * y + 0.5 * z)
    assert np.allclose(g[:, 0], 2, atol=1e-12)
    assert np.allclose(g[:, 1], -3, atol=1e-12)
    assert np.allclose(g[:, 2], 0.5, atol=1e-12)
    # 9/7/5-point interior stencils are exact for cubics; 3/2-point edges not
    g = oracle.grad_nospin(n, a, x ** 3)
    i = np.arange(n ** 3) % n
    inner = (i >= 2) & (i <= n - 3)
    assert np.allclose(g[inner, 0], 3 * x[inner] ** 2, rtol=1e-10)
    assert not np.allclose(g[i == 0, 0], 3 * x[i == 0] ** 2, rtol=1e-3)


def test_laplacian_edge_quirk():
    """derivative2 uses a first-derivative formula at pos 0 and n-1
    (differential_operators.cpp:562-578)."""
    n, a = 12, 5.5
    x, y, z, h = _xyz(n, a)
    lap = oracle.lap_nospin(n, a, x ** 2)
    i = np.arange(n ** 3) % n
    j = (np.arange(n ** 3) // n) % n
    k = np.arange(n ** 3) // n ** 2
    # y, z derivative2 of x^2 is 0 except the first-derivative edge formula,
    # which is also 0 for a function constant along the axis
    inner = (i >= 1) & (i <= n - 2)
    assert np.allclose(lap[inner], 2.0, rtol=1e-10)
    edge0 = i == 0
    expect = (x[edge0] + h) ** 2 - x[edge0] ** 2
    assert np.allclose(lap[edge0], expect / h, rtol=1e-12)


def _numpy_h(n, a, f, gradf, U, W, UC, X):
    """Independent restatement of the five Skyrme terms as array stencils."""
    h = 2 * a / (n - 1)
    ns = n ** 3
    psi = X.reshape(n, n, n, 2, order="C")  # [k][j][i][s]
    f3 = f.reshape(n, n, n)
    U3 = U.reshape(n, n, n) + (0 if UC is None else UC.reshape(n, n, n))
    g3 = [gradf[c * ns:(c + 1) * ns].reshape(n, n, n) for c in range(3)]
    W3 = [np.zeros((n, n, n)) if W is None else
          W[c * ns:(c + 1) * ns].reshape(n, n, n) for c in range(3)]

    def sh(v, ax, d):  # v at r + d e_ax, zero outside
        out = np.zeros_like(v)
        axis = 2 - ax  # array axes: 0 = k (z), 1 = j (y), 2 = i (x)
        src = [slice(None)] * v.ndim
        dst = [slice(None)] * v.ndim
        if d > 0:
            src[axis] = slice(d, None)
            dst[axis] = slice(None, -d)
        else:
            src[axis] = slice(None, d)
            dst[axis] = slice(-d, None)
        out[tuple(dst)] = v[tuple(src)]
        return out

    out = (U3 + 7.5 * f3 / h ** 2)[..., None] * psi
    sx = np.array([[0, 1], [1, 0]], complex)
    sy = np.array([[0, -1j], [1j, 0]])
    sz = np.array([[1, 0], [0, -1]], complex)
    for ax in range(3):
        L = (4 / 3) * (sh(psi, ax, 1) + sh(psi, ax, -1)) - (1 / 12) * (
            sh(psi, ax, 2) + sh(psi, ax, -2))
        out -= (f3 / h ** 2)[..., None] * L
        D = (8 * (sh(psi, ax, 1) - sh(psi, ax, -1)) -
             (sh(psi, ax, 2) - sh(psi, ax, -2))) / (12 * h)
        out += (-g3[ax])[..., None] * D
        Wx, Wy, Wz = W3
        if ax == 0:
            M = sy[None, None, None] * Wz[..., None, None] - \
                sz[None, None, None] * Wy[..., None, None]
        elif ax == 1:
            M = sz[None, None, None] * Wx[..., None, None] - \
                sx[None, None, None] * Wz[..., None, None]
        else:
            M = sx[None, None, None] * Wy[..., None, None] - \
                sy[None, None, None] * Wx[..., None, None]
        out += -1j * np.einsum("kjist,kjit->kjis", M, D)
    return out.reshape(-1)


@pytest.mark.parametrize("n,so,coul", [(6, True, False), (9, True, True),
                                       (8, False, False)])
def test_csr_matches_numpy_terms(n, so, coul):
    a = 0.5 * (n - 1) * 0.9
    f, gradf, U, W, UC = random_fields(n, 11 + n, so=so, coulomb=coul)
    H = oracle.Hamiltonian.skyrme(n, a, f, gradf, U, W, UC)
    X = random_block(2 * n ** 3, 2, 3)
    Y = H.apply(X)
    for c in range(2):
        ref = _numpy_h(n, a, f, gradf, U, W, UC, X[:, c])
        assert np.abs(Y[:, c] - ref).max() <= 1e-12 * np.abs(ref).max()


def test_csr_structure_and_hermiticity():
    n, a = 8, 3.5
    f, gradf, U, W, UC = random_fields(n, 5)
    H = oracle.Hamiltonian.skyrme(n, a, f, gradf, U, W)
    rp, col, val = H.csr()
    N = 2 * n ** 3
    assert rp[-1] == H.nnz()
    # interior rows: 1 diagonal + 12 same-spin kinetic + SO blocks; at most 26
    counts = np.diff(rp)
    assert counts.max() <= 26 and counts.min() >= 7
    for r in range(0, N, 97):
        assert np.all(np.diff(col[rp[r]:rp[r + 1]]) > 0)  # ascending columns
    # row-point fields make H non-Hermitian; constant f and W=0 restore it
    import scipy.sparse as sp
    M = sp.csr_matrix((val, col, rp), shape=(N, N))
    assert abs(M - M.conj().T).max() > 1e-6
    f0 = np.full(n ** 3, 20.7)
    H0 = oracle.Hamiltonian.skyrme(n, a, f0, np.zeros(3 * n ** 3), U)
    rp, col, val = H0.csr()
    M0 = sp.csr_matrix((val, col, rp), shape=(N, N))
    assert abs(M0 - M0.conj().T).max() < 1e-12


def test_woods_saxon_matches_skyrme_form():
    """build_matrix5p with WS terms equals the Skyrme stencil with constant
    f = hbar^2/2m, U = V_WS and W = ls grad V_SO (the form the GPU uses)."""
    n, a, A, Z = 10, 4.5, 16, 8
    H = oracle.Hamiltonian.woods_saxon(n, a, A, Z)
    X = random_block(2 * n ** 3, 2, 9)
    Y = H.apply(X)
    hbar, m = 197.327053, 938.91869
    x, y, z, h = _xyz(n, a)
    r = np.sqrt(x * x + y * y + z * z)
    R = 1.2 * A ** (1 / 3)
    U = -55.5 * (1 + 0.86 * (A - 2 * Z) / A) / (1 + np.exp((r - R) / 0.67))
    et = np.exp((r - R) / 0.67)
    sc = (55.5 / 0.67) * et / (1 + et) ** 2
    ls = -35.0 * (hbar * 0.5 / m) ** 2
    W = np.concatenate([ls * sc * x / r, ls * sc * y / r, ls * sc * z / r])
    f = np.full(n ** 3, hbar ** 2 / (2 * m))
    ref = _numpy_h(n, a, f, np.zeros(3 * n ** 3), U, W, None, X[:, 0])
    assert np.abs(Y[:, 0] - ref).max() <= 1e-11 * np.abs(ref).max()


def test_harmonic_oscillator_levels():
    """Known answer: constant f, U = m w^2 r^2 / 2 -> hbar w (N + 3/2)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    n, a = 24, 8.0
    hbar, m = 197.327053, 938.91869
    hw = 10.0
    x, y, z, h = _xyz(n, a)
    U = 0.5 * m * (hw / hbar) ** 2 * (x * x + y * y + z * z)
    f = np.full(n ** 3, hbar ** 2 / (2 * m))
    H = oracle.Hamiltonian.skyrme(n, a, f, np.zeros(3 * n ** 3), U)
    rp, col, val = H.csr()
    N = 2 * n ** 3
    M = sp.csr_matrix((val, col, rp), shape=(N, N))
    # deterministic start vector; the N=1 level is 6-fold degenerate, so ask
    # for more pairs than needed
    v0 = np.ones(N, dtype=complex) / np.sqrt(N)
    w = np.sort(sla.eigsh(M, k=12, sigma=0, which="LM", v0=v0, ncv=48,
                          tol=1e-10)[0].real)
    # Lanczos from one start vector returns one member of each exactly
    # degenerate (Kramers) multiplet: compare the distinct shells
    levels = np.unique(np.round(w, 1))
    assert np.allclose(levels[:3], [1.5 * hw, 2.5 * hw, 3.5 * hw], rtol=2e-3)


def test_heig_and_mgs_against_numpy():
    rng = np.random.default_rng(0)
    m = 17
    A = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
    A = A + A.conj().T
    w, V = oracle.heig(A)
    assert np.allclose(w, np.linalg.eigvalsh(A), atol=1e-12)
    assert np.abs(A @ V - V * w).max() < 1e-11
    Q = oracle.mgs(random_block(500, 6, 1))
    assert np.abs(Q.conj().T @ Q - np.eye(6)).max() < 1e-13


def test_gcg_converges_to_lowest_eigenpairs():
    """Many GCG iterations reproduce the lowest eigenvalues of a small H."""
    n, a = 8, 5.0
    f, gradf, U, W, UC = random_fields(n, 3)
    f0 = np.full(n ** 3, 20.7)
    H = oracle.Hamiltonian.skyrme(n, a, f0, np.zeros(3 * n ** 3), U, None)
    rp, col, val = H.csr()
    import scipy.sparse as sp
    N = 2 * n ** 3
    dense = sp.csr_matrix((val, col, rp), shape=(N, N)).toarray()
    ref = np.linalg.eigvalsh(dense)[:6]
    X0 = random_block(N, 6, 4)
    X, lam, info = H.gcg(X0, 6, max_iter=60, tol=1e-9, cg_steps=40,
                         cg_tol=1e-9)
    assert np.allclose(lam, ref, atol=1e-7)


def test_pcg_reduces_residual():
    n, a = 8, 4.0
    f, gradf, U, W, UC = random_fields(n, 8)
    H = oracle.Hamiltonian.skyrme(n, a, f, gradf, U, W)
    B = random_block(2 * n ** 3, 3, 2)
    X0 = np.zeros_like(B)
    shift = 80.0
    Wsol, steps = H.pcg(B, X0, shift, 200, 1e-10)
    R = B - H.apply(Wsol, shift)
    # row-point fields make H mildly non-Hermitian: CG still converges here
    assert (np.linalg.norm(R, axis=0) / np.linalg.norm(B, axis=0)).max() < 1e-6
    assert steps.max() <= 200


def _index_waves(n, m):
    """exp(2 pi i (m0 i + m1 j + m2 k) / n) on the lattice indices (x
    fastest) and its three index wave numbers."""
    ii = np.arange(n)
    K, J, I = np.meshgrid(ii, ii, ii, indexing="ij")
    ph = 2 * np.pi * (m[0] * I + m[1] * J + m[2] * K) / n
    return np.exp(1j * ph).ravel()


def test_lagrange_gradient_exact_on_band_limited_waves():
    """lagrangeFirstDerivative with the gradLagrange contraction is the
    derivative of the periodic trigonometric interpolant for odd n: exact
    (to rounding) on waves below the Nyquist index, both spins, all axes."""
    n, a = 11, 4.0
    h = 2 * a / (n - 1)
    m = (2, -3, 1)
    up = _index_waves(n, m)
    dn = 0.5 * _index_waves(n, (-1, 4, -2))
    psi = np.zeros(2 * n ** 3, np.complex128)
    psi[0::2], psi[1::2] = up, dn
    g = oracle.grad_lagrange(n, a, psi)
    for ax in range(3):
        want_up = 1j * 2 * np.pi * m[ax] / (n * h) * up
        want_dn = 1j * 2 * np.pi * (-1, 4, -2)[ax] / (n * h) * dn
        assert np.abs(g[ax, 0::2] - want_up).max() < 1e-12
        assert np.abs(g[ax, 1::2] - want_dn).max() < 1e-12


def test_lagrange_laplacian_exact_on_band_limited_waves():
    """lapLagrangeNoSpin (D D on each axis, summed) on a real wave: minus
    the squared wave numbers, for odd n."""
    n, a = 13, 5.0
    h = 2 * a / (n - 1)
    m = (1, 2, -4)
    rho = np.real(_index_waves(n, m)) + 0.3
    _, _, lap = oracle.lagrange_densities(
        n, a, np.zeros((2 * n ** 3, 1), np.complex128), rho)
    k2 = sum((2 * np.pi * mi / (n * h)) ** 2 for mi in m)
    assert np.abs(lap - (-k2) * (rho - 0.3)).max() < 1e-10


def test_lagrange_densities_from_the_gradient():
    """tau = sum |g|^2 and J_{mu nu} = Im(psi^* sigma_nu g_mu) summed over
    columns, restated in numpy from the oracle's Lagrange gradient."""
    n, a = 7, 3.0
    Phi = random_block(2 * n ** 3, 3, 17)
    tau, J9, _ = oracle.lagrange_densities(n, a, Phi)
    ns = n ** 3
    sig = [np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]),
           np.array([[1, 0], [0, -1]])]
    tw, Jw = np.zeros(ns), np.zeros((ns, 9))
    for c in range(Phi.shape[1]):
        psi = Phi[:, c]
        g = oracle.grad_lagrange(n, a, psi)
        P = psi.reshape(ns, 2)
        for mu in range(3):
            G = g[mu].reshape(ns, 2)
            tw += (np.abs(G) ** 2).sum(axis=1)
            for nu in range(3):
                Jw[:, mu * 3 + nu] += np.imag(
                    (P.conj() * (G @ sig[nu].T)).sum(axis=1))
    assert np.abs(tau - tw).max() < 1e-12 * np.abs(tw).max()
    assert np.abs(J9 - Jw).max() < 1e-12 * np.abs(Jw).max()


def test_shell_observables_of_a_p3half_state():
    """(x + iy) exp(-r^2 / 2b^2) spin up is l = 1, j = 3/2, mj = 3/2, odd:
    <L^2> = 2 hbar^2, <J^2> = 15/4 hbar^2, <Jz Jz> = 9/4 hbar^2,
    <L.S> = hbar^2 / 2 (finite-difference operators on a 25^3 lattice)."""
    import math
    n, a = 25, 7.2
    h = 2 * a / (n - 1)
    xs = -a + np.arange(n) * h
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    b = 1.7
    psi = np.zeros(2 * n ** 3, np.complex128)
    psi[0::2] = ((X + 1j * Y) * np.exp(-(X ** 2 + Y ** 2 + Z ** 2) /
                                       (2 * b * b))).ravel()
    psi /= math.sqrt(oracle.integral(n, a, np.abs(psi[0::2]) ** 2))
    L2, J2, JJ, par, LS = oracle.shell_observables(n, a, psi)[0]
    hb2 = 197.327053 ** 2
    assert abs(L2 / hb2 - 2.0) < 1e-3
    assert abs(J2 / hb2 - 3.75) < 1e-3
    assert abs(JJ / hb2 - 2.25) < 1e-3
    assert abs(LS / hb2 - 0.5) < 1e-3
    assert par < 0
    from nuclearcgm_gb300 import output
    assert output.classify([[L2, J2, JJ, par, LS]])[0][:3] == (1.0, 1.5, 1.5)


def test_multipole_constraint_joins_at_iteration_one():
    """A general multipole constraint (MultipoleConstraint) is added at HF
    iteration 1: iteration 0 is unchanged; from iteration 1 E_HF carries the
    constraint energy C (Q - target)^2 + lambda (Q - target), about
    0.01 MeV at first (C = 0.01 / (Q - target)^2)."""
    from nuclearcgm_gb300 import config
    data = {"functional": "SLy4", "nucleus": {"A": 16, "Z": 8},
            "box": {"boxSize": 14.0, "axisMeshPoints": 10},
            "maxIterations": 3, "energyTol": 0.0}
    r0, o0 = oracle.hf_run(config.from_input(data))
    r1, o1 = oracle.hf_run(config.from_input(
        dict(data, constraints=[{"l": 2, "m": 0, "target": 25.0}])))
    assert np.array_equal(o0["energies"][0], o1["energies"][0])
    assert np.all(np.isfinite(o1["energies"]))
    d = abs(o1["energies"][1, 1] - o0["energies"][1, 1])
    assert 1e-3 < d < 0.1


def test_hfb_switched_off_species_occupies_particle_number_states():
    """After a species' HFB pairing energy drops to zero the run switches
    its pairing off and occupies phi * nullOcc(particles)
    (iteration_data.cpp:290-294, 319-323). With a basis larger than the
    particle number (20 states for 8 nucleons here) the reference's release
    build keeps the first `particles` columns: the densities must still
    integrate to N and Z, not to the basis size."""
    from nuclearcgm_gb300 import config
    n, box = 10, 16.5
    data = {"functional": "SKMstar", "nucleus": {"A": 16, "Z": 8},
            "box": {"boxSize": box, "axisMeshPoints": n},
            "pairing": {"type": "HFB", "HFbasisSize": 20, "V0": 100.0,
                        "window": 5.0},
            "maxIterations": 12, "energyTol": 0.0}
    res, out = oracle.hf_run(config.from_input(data))
    assert res.E_pair_n == 0.0 and res.E_pair_p == 0.0
    h = box / (n - 1)
    w = np.ones(n)
    w[0] = w[-1] = 0.5
    wt = (w[:, None, None] * w[None, :, None] * w[None, None, :]).ravel()
    for q in ("rho_n", "rho_p"):
        assert abs((out[q] * wt).sum() * h ** 3 - 8.0) < 1e-8
    # the 20 basis states are all still solved for
    assert out["spe_n"].shape == (20,) and np.all(np.diff(out["spe_n"]) >= 0)
