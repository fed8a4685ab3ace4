"""Seeded synthetic inputs of the standalone H.X / GCG-step workload.

40^3 lattice, h = 0.5 fm (a = 9.75 fm), a block of 64 complex 2-spinors with
i.i.d. N(0,1) real and imaginary parts, orthonormalised in FP64, and fields:
  U(r)   = clip(-sum_8 D_k exp(-|r-c_k|^2/w_k^2), -60, 0),
           D_k ~ U[0,60] MeV, w_k ~ U[1.5,3] fm, c_k ~ U[-a/2,a/2]^3  (seed 2)
  f(r)   = 20.7 (1 - 0.3 g(r)) MeV fm^2, g a Gaussian sum scaled to [0,1]
           (seed 3), grad f analytic
  W(r)   = kappa grad G(r), G a Gaussian sum (seed 4), max|W| = 10 MeV fm.
Random numbers come from splitmix64 with Box-Muller, so the inputs are the
same on every machine.
"""
from __future__ import annotations

import numpy as np

_M64 = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed: int):
        self.state = np.uint64(seed & _M64)

    def next_u64(self, count: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            inc = np.uint64(0x9E3779B97F4A7C15)
            steps = (np.arange(1, count + 1, dtype=np.uint64) * inc)
            z = self.state + steps
            self.state = z[-1] if count else self.state
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        return z

    def uniform(self, count: int) -> np.ndarray:
        """Doubles in (0, 1) from the top 53 bits."""
        u = (self.next_u64(count) >> np.uint64(11)).astype(np.float64)
        return (u + 0.5) * (1.0 / 9007199254740992.0)

    def normal(self, count: int) -> np.ndarray:
        m = (count + 1) // 2
        u1, u2 = self.uniform(m), self.uniform(m)
        r = np.sqrt(-2.0 * np.log(u1))
        z = np.concatenate([r * np.cos(2 * np.pi * u2),
                            r * np.sin(2 * np.pi * u2)])
        return z[:count]


def lattice(n: int, a: float):
    h = 2.0 * a / (n - 1)
    xs = -a + np.arange(n) * h
    # i-fastest flattening: index = i + n (j + n k)
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    return X.ravel(), Y.ravel(), Z.ravel(), h


def _gauss_sum(rng, x, y, z, a, count, dmin, dmax, wmin, wmax):
    D = dmin + (dmax - dmin) * rng.uniform(count)
    w = wmin + (wmax - wmin) * rng.uniform(count)
    c = (-a / 2) + a * rng.uniform(3 * count).reshape(count, 3)
    G = np.zeros_like(x)
    gx, gy, gz = np.zeros_like(x), np.zeros_like(x), np.zeros_like(x)
    for k in range(count):
        dx, dy, dz = x - c[k, 0], y - c[k, 1], z - c[k, 2]
        e = D[k] * np.exp(-(dx * dx + dy * dy + dz * dz) / w[k] ** 2)
        G += e
        gx += e * (-2 * dx / w[k] ** 2)
        gy += e * (-2 * dy / w[k] ** 2)
        gz += e * (-2 * dz / w[k] ** 2)
    return G, np.stack([gx, gy, gz], axis=1)


def fields(n=40, h=0.5):
    """(a, f, gradf[n^3 x 3], U, W[n^3 x 3]) of the synthetic workload."""
    a = 0.5 * (n - 1) * h
    x, y, z, _ = lattice(n, a)
    G, _ = _gauss_sum(SplitMix64(2), x, y, z, a, 8, 0.0, 60.0, 1.5, 3.0)
    U = np.clip(-G, -60.0, 0.0)
    g, dg = _gauss_sum(SplitMix64(3), x, y, z, a, 8, 0.0, 1.0, 1.5, 3.0)
    gmax = g.max()
    f = 20.7 * (1.0 - 0.3 * g / gmax)
    gradf = -20.7 * 0.3 * dg / gmax
    Gs, dG = _gauss_sum(SplitMix64(4), x, y, z, a, 8, 0.0, 1.0, 1.5, 3.0)
    kappa = 10.0 / np.sqrt((dG ** 2).sum(axis=1)).max()
    W = kappa * dG
    return a, f, gradf, U, W


def orthonormal_block(N: int, ncols: int, seed: int = 1) -> np.ndarray:
    """N x ncols complex block with N(0,1) parts, CholQR2-orthonormalised in
    FP64; Fortran order (Eigen layout)."""
    rng = SplitMix64(seed)
    v = rng.normal(2 * N * ncols)
    X = (v[0::2] + 1j * v[1::2]).reshape(ncols, N).T
    X = np.asfortranarray(X)
    for _ in range(2):
        G = X.conj().T @ X
        L = np.linalg.cholesky(G)
        X = np.asfortranarray(np.linalg.solve(L, X.T.conj()).conj().T)
    return X


def hx_bytes(n: int, ncols: int, real_bytes: int) -> int:
    """Algorithmic bytes of one H.X: X read once + Y written once, plus the 8
    per-point field values read once."""
    ns = n ** 3
    return ns * ncols * (2 * 2 * real_bytes) * 2 + ns * 8 * real_bytes
