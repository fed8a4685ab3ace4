"""Test infrastructure: ctypes loader for the FP64 CPU oracle.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker. The oracle is a restatement of the
reference algorithm and is "parity unpinned" against the reference binary
(see ncgm_oracle.h).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libncgm_oracle.so")
_lib = None


def build(force=False):
    """Compile the oracle with its Makefile (seconds)."""
    if force or not os.path.exists(LIB) or any(
            os.path.getmtime(os.path.join(HERE, f)) > os.path.getmtime(LIB)
            for f in os.listdir(HERE) if f.endswith((".cpp", ".hpp", ".h"))):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        vp, i, d = C.c_void_p, C.c_int, C.c_double
        sig = {
            "orc_h_build_skyrme": ([i, d, vp, vp, vp, vp, vp], vp),
            "orc_h_build_ws": ([i, d, i, i, d, d, d, d, d, d, d, i], vp),
            "orc_h_nnz": ([vp], C.c_longlong),
            "orc_h_export": ([vp, vp, vp, vp], None),
            "orc_h_apply": ([vp, vp, vp, i, d], None),
            "orc_h_diag": ([vp, vp], None),
            "orc_h_free": ([vp], None),
            "orc_gcg": ([vp, vp, i, vp, i, i, d, i, d, i, d, i, vp, vp, vp], i),
            "orc_pcg": ([vp, vp, vp, vp, i, d, i, d, vp], None),
            "orc_mgs": ([vp, C.c_longlong, i], None),
            "orc_heig": ([vp, i, vp, vp], i),
            "orc_density": ([i, d, vp, i, vp], None),
            "orc_kinetic_density": ([i, d, vp, i, vp], None),
            "orc_so_density": ([i, d, vp, i, vp], None),
            "orc_divj": ([i, d, vp, i, vp], None),
            "orc_grad_nospin": ([i, d, vp, vp], None),
            "orc_lap_nospin": ([i, d, vp, vp], None),
            "orc_grad_spinor": ([i, d, vp, vp], None),
            "orc_grad_lagrange": ([i, d, vp, vp], None),
            "orc_lagrange_densities": ([i, d, vp, i, vp, vp, vp, vp], None),
            "orc_integral": ([i, d, vp], d),
            "orc_poisson": ([i, d, vp, i, vp, vp], i),
            "orc_ho_guess": ([i, d, i, d, d, vp], None),
            "orc_hf_run": ([vp, vp, vp, vp, vp, vp, vp, i], i),
            "orc_hf_run_ex": ([vp, vp, vp, vp, vp, vp, vp, vp, i], i),
            "orc_shell_observables": ([i, d, vp, i, vp], None),
            "orc_state_run": ([vp, vp, vp, i, vp, vp, i, i, i, vp, vp, vp,
                               vp], i),
        }
        for name, (a, r) in sig.items():
            f = getattr(_lib, name)
            f.argtypes = a
            f.restype = r
    return _lib


def _p(x):
    return None if x is None else x.ctypes.data


def _c(x, dtype):
    return None if x is None else np.ascontiguousarray(x, dtype=dtype)


def _cmat(X):
    """Complex column-major (Eigen layout) view as interleaved doubles."""
    return np.asfortranarray(X, dtype=np.complex128)


class Hamiltonian:
    """Assembled CSR Hamiltonian of the oracle."""

    def __init__(self, handle, n, a):
        self.h, self.n, self.a = handle, n, a
        self.N = 2 * n ** 3

    @classmethod
    def skyrme(cls, n, a, f, gradf, U, W=None, UC=None):
        args = [_c(f, np.float64), _c(gradf, np.float64), _c(U, np.float64),
                _c(W, np.float64), _c(UC, np.float64)]
        h = lib().orc_h_build_skyrme(n, a, *[_p(x) for x in args])
        return cls(h, n, a)

    @classmethod
    def woods_saxon(cls, n, a, A, Z, V0=55.5, r0=1.2, diff=0.67, kappa=0.86,
                    beta=0.0, beta3=0.0, so_V0=55.5, spin_orbit=True):
        h = lib().orc_h_build_ws(n, a, A, Z, V0, r0, diff, kappa, beta, beta3,
                                 so_V0, int(spin_orbit))
        return cls(h, n, a)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_h_free(self.h)
            self.h = None

    def nnz(self):
        return lib().orc_h_nnz(self.h)

    def csr(self):
        nnz = self.nnz()
        rp = np.zeros(self.N + 1, np.int64)
        col = np.zeros(nnz, np.int32)
        val = np.zeros(nnz, np.complex128)
        lib().orc_h_export(self.h, _p(rp), _p(col), _p(val))
        return rp, col, val

    def diag(self):
        d = np.zeros(self.N, np.complex128)
        lib().orc_h_diag(self.h, _p(d))
        return d

    def apply(self, X, shift=0.0):
        X = _cmat(X)
        ncols = 1 if X.ndim == 1 else X.shape[1]
        Y = np.zeros_like(X)
        lib().orc_h_apply(self.h, _p(X), _p(Y), ncols, shift)
        return Y

    def gcg(self, X_init, nev, ConjDir=None, shift=0.0, max_iter=1, tol=1e-6,
            cg_steps=80, cg_tol=1e-5, ordering=1):
        X_init = _cmat(X_init)
        P = None if ConjDir is None else _cmat(ConjDir)
        Xo = np.zeros((self.N, nev), np.complex128, order="F")
        lam = np.zeros(nev)
        steps = C.c_int(0)
        kept = lib().orc_gcg(self.h, _p(X_init), X_init.shape[1], _p(P),
                             0 if P is None else P.shape[1], nev, shift,
                             max_iter, tol, cg_steps, cg_tol, ordering,
                             _p(Xo), _p(lam), C.addressof(steps))
        return Xo, lam, {"basis_cols": kept, "pcg_steps": steps.value}

    def pcg(self, B, X0, shift, max_steps, tol):
        B, X0 = _cmat(B), _cmat(X0)
        W = np.zeros_like(B)
        ncols = B.shape[1]
        steps = np.zeros(ncols, np.int32)
        lib().orc_pcg(self.h, _p(B), _p(X0), _p(W), ncols, shift, max_steps,
                      tol, _p(steps))
        return W, steps


def mgs(V):
    V = _cmat(V).copy(order="F")
    lib().orc_mgs(_p(V), V.shape[0], V.shape[1])
    return V


def heig(A):
    A = _cmat(A)
    m = A.shape[0]
    w = np.zeros(m)
    V = np.zeros((m, m), np.complex128, order="F")
    lib().orc_heig(_p(A), m, _p(w), _p(V))
    return w, V


def _lat(fn, n, a, psi, out_shape):
    psi = _cmat(psi)
    ncols = 1 if psi.ndim == 1 else psi.shape[1]
    out = np.zeros(out_shape)
    fn(n, a, _p(psi), ncols, _p(out))
    return out


def density(n, a, psi):
    return _lat(lib().orc_density, n, a, psi, n ** 3)


def kinetic_density(n, a, psi):
    return _lat(lib().orc_kinetic_density, n, a, psi, n ** 3)


def so_density(n, a, psi):
    """J_{mu nu}, n^3 x 9 column-major (col mu*3+nu)."""
    return _lat(lib().orc_so_density, n, a, psi, 9 * n ** 3).reshape(
        9, n ** 3).T


def divj(n, a, psi):
    return _lat(lib().orc_divj, n, a, psi, n ** 3)


def grad_nospin(n, a, v):
    v = _c(v, np.float64)
    out = np.zeros(3 * n ** 3)
    lib().orc_grad_nospin(n, a, _p(v), _p(out))
    return out.reshape(3, n ** 3).T


def lap_nospin(n, a, v):
    v = _c(v, np.float64)
    out = np.zeros(n ** 3)
    lib().orc_lap_nospin(n, a, _p(v), _p(out))
    return out


def grad_spinor(n, a, psi):
    psi = np.ascontiguousarray(psi, np.complex128)
    out = np.zeros((3, 2 * n ** 3), np.complex128)
    lib().orc_grad_spinor(n, a, _p(psi), _p(out))
    return out


def grad_lagrange(n, a, psi):
    """Operators::gradLagrange of one spinor: (3, 2 n^3) complex."""
    psi = np.ascontiguousarray(psi, np.complex128)
    out = np.zeros((3, 2 * n ** 3), np.complex128)
    lib().orc_grad_lagrange(n, a, _p(psi), _p(out))
    return out


def lagrange_densities(n, a, psi, rho=None):
    """tau (n^3), J_{mu nu} (n^3 x 9) and, with rho, the Laplacian of rho,
    all with the Lagrange-mesh derivatives of the output step."""
    psi = _cmat(psi)
    ncols = 1 if psi.ndim == 1 else psi.shape[1]
    ns = n ** 3
    tau, J9 = np.zeros(ns), np.zeros(9 * ns)
    lap = np.zeros(ns) if rho is not None else None
    r = _c(rho, np.float64) if rho is not None else None
    lib().orc_lagrange_densities(n, a, _p(psi), ncols,
                                 _p(r) if r is not None else None, _p(tau),
                                 _p(J9), _p(lap) if lap is not None else None)
    return tau, J9.reshape(9, ns).T, lap


def integral(n, a, v):
    return lib().orc_integral(n, a, _p(_c(v, np.float64)))


def poisson(n, a, rhoP, Z, U_guess=None):
    rhoP = _c(rhoP, np.float64)
    U = np.zeros(n ** 3)
    g = _c(U_guess, np.float64)
    it = lib().orc_poisson(n, a, _p(rhoP), Z, _p(g), _p(U))
    return U, it


def ho_guess(n, a, nev, b, beta=0.0):
    out = np.zeros((2 * n ** 3, nev), np.complex128, order="F")
    lib().orc_ho_guess(n, a, nev, b, beta, _p(out))
    return out


def shell_observables(n, a, psi):
    """orc_shell_observables: (ncols, 5) as ncgm_shell_observables."""
    psi = _cmat(psi)
    if psi.ndim == 1:
        psi = psi.reshape(-1, 1, order="F")
    obs = np.zeros((psi.shape[1], 5))
    lib().orc_shell_observables(n, a, _p(psi), psi.shape[1], _p(obs))
    return obs


def hf_run_ex(cfg, verbose=False):
    """orc_hf_run_ex: hf_run plus the output step's arrays and energy table
    (the keys of nuclearcgm_gb300.hf_run(cfg, outputs=True))."""
    from nuclearcgm_gb300 import abi, config
    res = abi.HFResult()
    on, op = config.orbital_counts(cfg)
    ns = cfg.n ** 3
    N = 2 * ns
    arr = {"spe_n": np.zeros(on), "spe_p": np.zeros(op),
           "rho_n": np.zeros(ns), "rho_p": np.zeros(ns)}
    en = np.zeros((max(cfg.max_iterations, 1), 2))
    extra = {"orbitals_n": np.zeros((N, on), np.complex128, order="F"),
             "orbitals_p": np.zeros((N, op), np.complex128, order="F"),
             "tau_n": np.zeros(ns), "tau_p": np.zeros(ns),
             "grad_rho_n": np.zeros(3 * ns), "grad_rho_p": np.zeros(3 * ns),
             "U_n": np.zeros(ns), "U_p": np.zeros(ns)}
    out = abi.HFOutputs(**{k: v.ctypes.data for k, v in extra.items()})
    lib().orc_hf_run_ex(C.addressof(cfg), C.addressof(res),
                        _p(arr["spe_n"]), _p(arr["spe_p"]), _p(arr["rho_n"]),
                        _p(arr["rho_p"]), _p(en), C.addressof(out),
                        int(verbose))
    for q in ("n", "p"):
        extra["grad_rho_" + q] = extra["grad_rho_" + q].reshape(3, ns).T
    arr.update(extra)
    arr["terms"] = np.array(out.terms[:])
    arr["constraints_energy"] = out.constraints_energy
    arr["energies"] = en[:res.iterations]
    return res, arr


def hf_run(cfg, verbose=False):
    """orc_hf_run on an abi.HFConfig. Returns (result, dict of arrays)."""
    from nuclearcgm_gb300 import abi, config
    res = abi.HFResult()
    on, op = config.orbital_counts(cfg)
    ns = cfg.n ** 3
    spe_n, spe_p = np.zeros(on), np.zeros(op)
    rho_n, rho_p = np.zeros(ns), np.zeros(ns)
    en = np.zeros((max(cfg.max_iterations, 1), 2))
    lib().orc_hf_run(C.addressof(cfg), C.addressof(res), _p(spe_n), _p(spe_p),
                     _p(rho_n), _p(rho_p), _p(en), int(verbose))
    en = en[:res.iterations]
    return res, {"spe_n": spe_n, "spe_p": spe_p, "rho_n": rho_n,
                 "rho_p": rho_p, "energies": en}


def state_run(cfg, neutrons, protons, calls, flags=1, new_levels=None):
    """The state-update counterpart of ncgm_state_* (orc_state_run):
    `calls` updates of IterationData from the same eigenpairs, then the
    energies with new_levels (default: the same levels). Returns a dict of
    per-species f, gradf, U, W, UC, rho, tau (suffix _n / _p) and E_int,
    E_HF."""
    (Xn, en), (Xp, ep) = neutrons, protons
    Xn = np.asfortranarray(Xn, dtype=np.complex128)
    Xp = np.asfortranarray(Xp, dtype=np.complex128)
    en = np.ascontiguousarray(en, dtype=np.float64)
    ep = np.ascontiguousarray(ep, dtype=np.float64)
    en2, ep2 = (en, ep) if new_levels is None else (
        np.ascontiguousarray(new_levels[0], dtype=np.float64),
        np.ascontiguousarray(new_levels[1], dtype=np.float64))
    ns = cfg.n ** 3
    out = np.zeros(22 * ns)
    E = np.zeros(2)
    rc = lib().orc_state_run(C.byref(cfg), Xn.ctypes.data, en.ctypes.data,
                             Xn.shape[1], Xp.ctypes.data, ep.ctypes.data,
                             Xp.shape[1], int(calls), int(flags),
                             en2.ctypes.data, ep2.ctypes.data,
                             out.ctypes.data, E.ctypes.data)
    if rc != 0:
        raise RuntimeError("orc_state_run failed: %d" % rc)
    res = {"E_int": E[0], "E_HF": E[1]}
    o = 0
    for q in ("n", "p"):
        for name, k in (("f", 1), ("gradf", 3), ("U", 1), ("W", 3),
                        ("UC", 1), ("rho", 1), ("tau", 1)):
            res[name + "_" + q] = out[o:o + k * ns]
            o += k * ns
    return res
