"""GPU parity of the lattice density kernel and the Coulomb Poisson solve
against the oracle."""
import ctypes as C

import numpy as np
import pytest

import nuclearcgm_gb300 as ng
from conftest import random_block
from nuclearcgm_gb300 import abi
from oracle import oracle

pytestmark = pytest.mark.gpu


def _dens(ctx, Phi):
    n = ctx.grid.n
    ns = n ** 3
    rho, tau, divj = np.zeros(ns), np.zeros(ns), np.zeros(ns)
    J9 = np.zeros(9 * ns)
    Phi = np.asfortranarray(Phi, dtype=np.complex128)
    ng._check(ng.load().ncgm_densities(ctx.h, Phi.ctypes.data, Phi.shape[1],
                                       rho.ctypes.data, tau.ctypes.data,
                                       J9.ctypes.data, divj.ctypes.data))
    return rho, tau, J9.reshape(9, ns).T, divj


@pytest.mark.parametrize("n", [8, 11, 16])
def test_densities_match_oracle(n):
    a = 0.5 * (n - 1) * 0.8
    ctx = ng.Context(ng.Grid(n, a), 8)
    Phi = random_block(2 * n ** 3, 5, n) * 0.1
    rho, tau, J9, dj = _dens(ctx, Phi)
    for got, ref in ((rho, oracle.density(n, a, Phi)),
                     (tau, oracle.kinetic_density(n, a, Phi)),
                     (J9, oracle.so_density(n, a, Phi)),
                     (dj, oracle.divj(n, a, Phi))):
        assert np.abs(got - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1e-30)


@pytest.mark.parametrize("n", [8, 11, 16])
def test_lagrange_densities_match_oracle(n):
    """The output step's Lagrange-mesh tau, J_{mu nu} and Laplacian of rho
    (ncgm_lagrange_densities) against the oracle's restatement."""
    a = 0.5 * (n - 1) * 0.8
    ctx = ng.Context(ng.Grid(n, a), 8)
    Phi = np.asfortranarray(random_block(2 * n ** 3, 5, 2 * n) * 0.1)
    ns = n ** 3
    rho = oracle.density(n, a, Phi)
    tau, J9, lap = np.zeros(ns), np.zeros(9 * ns), np.zeros(ns)
    ng._check(ng.load().ncgm_lagrange_densities(
        ctx.h, Phi.ctypes.data, Phi.shape[1], rho.ctypes.data,
        tau.ctypes.data, J9.ctypes.data, lap.ctypes.data))
    tr, Jr, lr = oracle.lagrange_densities(n, a, Phi, rho)
    for got, ref in ((tau, tr), (J9.reshape(9, ns).T, Jr), (lap, lr)):
        assert np.abs(got - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1e-30)
    # without rho the Laplacian is skipped; tau and J are unchanged
    t2, J2 = np.zeros(ns), np.zeros(9 * ns)
    ng._check(ng.load().ncgm_lagrange_densities(
        ctx.h, Phi.ctypes.data, Phi.shape[1], None, t2.ctypes.data,
        J2.ctypes.data, None))
    assert np.array_equal(t2, tau) and np.array_equal(J2, J9)
    # rho without lap is an argument error
    assert ng.load().ncgm_lagrange_densities(
        ctx.h, Phi.ctypes.data, Phi.shape[1], rho.ctypes.data,
        t2.ctypes.data, J2.ctypes.data, None) == abi.NCGM_OK + 1
    ctx.close()


def _gauss_rho(n, a, Z, w=2.5, shift=(0.3, -0.2, 0.5), zfac=1.3):
    h = 2 * a / (n - 1)
    xs = -a + np.arange(n) * h
    Zg, Yg, Xg = np.meshgrid(xs, xs, xs, indexing="ij")
    r2 = ((Xg - shift[0]) ** 2 + (Yg - shift[1]) ** 2 +
          zfac * (Zg - shift[2]) ** 2)
    rho = np.exp(-r2 / w ** 2).ravel()
    return rho * Z / oracle.integral(n, a, rho)


@pytest.mark.parametrize("n", [10, 16, 24])
def test_poisson_matches_oracle(n):
    a = 0.5 * (n - 1) * 0.7
    Z = 8
    rho = _gauss_rho(n, a, Z)
    ctx = ng.Context(ng.Grid(n, a), 2)
    ns = n ** 3
    U, UC = np.zeros(ns), np.zeros(ns)
    its = C.c_int(0)
    ng._check(ng.load().ncgm_poisson(ctx.h, rho.ctypes.data, Z, None,
                                     U.ctypes.data, UC.ctypes.data,
                                     C.byref(its)))
    Uref, _ = oracle.poisson(n, a, rho, Z)
    assert np.abs(U - Uref).max() <= 1e-9 * np.abs(Uref).max()
    # Slater exchange added to the direct potential
    ex = -1.43996446 * (3 / np.pi) ** (1 / 3) * rho ** (1 / 3)
    assert np.allclose(UC, U + ex, rtol=1e-12, atol=1e-12)
    # warm start from the solution converges immediately to the same field
    U2 = np.zeros(ns)
    ng._check(ng.load().ncgm_poisson(ctx.h, rho.ctypes.data, Z,
                                     U.ctypes.data, U2.ctypes.data, None,
                                     C.byref(its)))
    assert np.abs(U2 - Uref).max() <= 1e-9 * np.abs(Uref).max()


def test_poisson_spherical_charge_known_answer():
    """Known answer: a spherical Gaussian charge has U = e^2 Z erf(r/w) / r;
    the lattice solution matches it to the discretisation error."""
    from math import erf
    n, a, Z, w = 24, 11.5, 20, 2.0
    rho = _gauss_rho(n, a, Z, w=w, shift=(0.0, 0.0, 0.0), zfac=1.0)
    ctx = ng.Context(ng.Grid(n, a), 2)
    U = np.zeros(n ** 3)
    ng._check(ng.load().ncgm_poisson(ctx.h, rho.ctypes.data, Z, None,
                                     U.ctypes.data, None, None))
    h = 2 * a / (n - 1)
    xs = -a + np.arange(n) * h
    m = n // 2
    for (i, j, k), rel in (((0, m, m), 1e-3), ((m, m, 0), 1e-3),
                           ((3, m, m), 1e-3), ((m, m, m), 5e-3)):
        r = np.sqrt(xs[i] ** 2 + xs[j] ** 2 + xs[k] ** 2)
        exact = 1.43996446 * Z * erf(r / w) / r
        assert abs(U[i + n * (j + n * k)] - exact) < rel * exact


@pytest.mark.parametrize("n", [12, 30, 37])
def test_poisson_fast_solver_matches_cg(monkeypatch, n):
    """The separable direct inverse (default) and the plain CG path
    (NCGM_POISSON_FAST=0) reach the same 1e-13 residual: the potentials agree
    to ~1e-12, the direct solve in one or two refinement steps."""
    a = 0.5 * (n - 1) * 0.6
    Z = 20
    rho = _gauss_rho(n, a, Z)
    ctx = ng.Context(ng.Grid(n, a), 2)
    ns = n ** 3
    Uf, Uc = np.zeros(ns), np.zeros(ns)
    itf, itc = C.c_int(0), C.c_int(0)
    ng._check(ng.load().ncgm_poisson(ctx.h, rho.ctypes.data, Z, None,
                                     Uf.ctypes.data, None, C.byref(itf)))
    monkeypatch.setenv("NCGM_POISSON_FAST", "0")
    ng._check(ng.load().ncgm_poisson(ctx.h, rho.ctypes.data, Z, None,
                                     Uc.ctypes.data, None, C.byref(itc)))
    print("n=%d: fast solver %d steps, CG %d iterations, max diff %.2e" % (
        n, itf.value, itc.value, np.abs(Uf - Uc).max() / np.abs(Uc).max()))
    assert itf.value <= 3
    assert np.abs(Uf - Uc).max() <= 1e-11 * np.abs(Uc).max()
