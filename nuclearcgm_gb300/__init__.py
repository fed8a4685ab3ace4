"""nuclearcgm_gb300: GB300-native (sm_103a) build of the nuclearcgm
self-consistent lattice hot path.

The compute lives in the in-tree CUDA library libncgm.so (C ABI in
include/ncgm.h). This package is the host-side mirror of the reference's
interfaces for the path:

  Grid                      <- Grid (include/grid.hpp)
  Hamiltonian               <- Hamiltonian + Potential terms
                               (include/hamiltonian.hpp, include/potential.hpp)
  gcgm_complex_no_B_lock    <- include/solver.hpp:43-47
  solve                     <- Utilities::solve (include/util/utilities.hpp)
  hf_run                    <- the HF(B) loop of main() (src/main.cpp)

There is no CPU fallback: if libncgm.so is missing or no CUDA device is
visible, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi, config

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libncgm.so")
_lib = None


class NcgmError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (abi.STATUS.get(status, status), msg))
        self.status = status


def load():
    """Load libncgm.so (built by __graft_entry__.build()). Raises if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NcgmError(abi.NCGM_OK + 2,
                            "libncgm.so not built: run __graft_entry__.build()")
        _lib = abi.bind(C.CDLL(LIB_PATH))
    return _lib


def _check(status):
    if status != abi.NCGM_OK:
        raise NcgmError(status, load().ncgm_last_error().decode())


def _ptr(x):
    """Raw address of a numpy array or a torch tensor (host or device)."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data


class Grid:
    """Grid(n, a): x_i = -a + i h, h = 2a/(n-1) (src/grid/grid.cpp:7-41)."""

    def __init__(self, n: int, a: float):
        if n < 2:
            raise ValueError("Grid error: n must be >= 2. Received n = %d" % n)
        self.n, self.a = int(n), float(a)
        self.h = 2.0 * a / (n - 1)
        self.xs = -a + np.arange(n) * self.h

    def idx(self, i, j, k, s):
        return s + 2 * (i + self.n * (j + self.n * k))

    def idx_nospin(self, i, j, k):
        return i + self.n * (j + self.n * k)

    @property
    def total_spatial_points(self):
        return self.n ** 3

    @property
    def total_points(self):
        return 2 * self.n ** 3

    def dV(self):
        return self.h ** 3


class Context:
    """Device context for one lattice (ncgm_create / ncgm_destroy)."""

    def __init__(self, grid: Grid, max_cols: int):
        self.grid = grid
        self.max_cols = max_cols
        h = C.c_void_p()
        _check(load().ncgm_create(C.byref(h), grid.n, grid.a, max_cols, 0))
        self.h = h

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            load().ncgm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _f64(x, n=None):
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return x
    a = np.ascontiguousarray(x, dtype=np.float64)
    if n is not None and a.size != n:
        raise ValueError("expected %d values, got %d" % (n, a.size))
    return a


class Hamiltonian:
    """Matrix-free H for one species on a Context.

    Replaces Hamiltonian(grid, terms).buildMatrix() with the Skyrme term list
    (src/hamiltonian/hamiltonian.cpp:303-372): the fields are uploaded and
    H.X is applied by the CUDA stencil. `apply` accepts (N, ncols) complex128
    arrays in the reference's Eigen layout (column-major) or device tensors.
    """

    def __init__(self, ctx: Context, species: int = abi.NEUTRON):
        self.ctx, self.species = ctx, species

    def set_fields(self, f, gradf, U, W=None, UC=None):
        ns = self.ctx.grid.n ** 3
        args = [_f64(f, ns), _f64(gradf, 3 * ns), _f64(U, ns),
                _f64(W, 3 * ns), _f64(UC, ns)]
        self._keep = args
        _check(load().ncgm_set_fields(self.ctx.h, self.species,
                                      *[_ptr(a) for a in args]))
        return self

    def set_woods_saxon(self, A, Z, V0=55.5, r0=1.2, diff=0.67, kappa=0.86,
                        beta=0.0, beta3=0.0, so_V0=55.5, spin_orbit=True):
        """Woods-Saxon guess H (Hamiltonian::build_matrix5p with the deformed
        WS and WS spin-orbit terms, src/main.cpp:72-86)."""
        _check(load().ncgm_set_woods_saxon(self.ctx.h, self.species, A, Z, V0,
                                           r0, diff, kappa, beta, beta3,
                                           so_V0, int(spin_orbit)))
        return self

    def apply(self, X, precision=abi.FP64):
        if hasattr(X, "data_ptr"):
            import torch
            # device tensors: (ncols, N) row-major == (N, ncols) Eigen layout
            Y = torch.empty_like(X)
            ncols = 1 if X.dim() == 1 else X.shape[0]
            _check(load().ncgm_apply_h(self.ctx.h, self.species, X.data_ptr(),
                                       Y.data_ptr(), ncols, precision))
            return Y
        X = np.asfortranarray(X, dtype=np.complex128)
        ncols = 1 if X.ndim == 1 else X.shape[1]
        Y = np.empty_like(X)
        _check(load().ncgm_apply_h(self.ctx.h, self.species, X.ctypes.data,
                                   Y.ctypes.data, ncols, precision))
        return Y

    def gcg(self, X_init, nev, ConjDir=None, params: abi.GcgParams = None):
        """gcgm_complex_no_B_lock (src/solver/solver.cpp:642-959)."""
        if params is None:
            params = config._gcg(config.HF_GCG)
        X_init = np.asfortranarray(X_init, dtype=np.complex128)
        P = None if ConjDir is None else np.asfortranarray(
            ConjDir, dtype=np.complex128)
        N = X_init.shape[0]
        Xo = np.zeros((N, nev), np.complex128, order="F")
        lam = np.zeros(nev)
        st = abi.GcgStats()
        _check(load().ncgm_gcg(self.ctx.h, self.species, X_init.ctypes.data,
                               X_init.shape[1], _ptr(P),
                               0 if P is None else P.shape[1], nev,
                               C.byref(params), Xo.ctypes.data, lam.ctypes.data,
                               C.byref(st)))
        return Xo, lam, st


def gcgm_complex_no_B_lock(H: Hamiltonian, X_initial, ConjDir, nev,
                           shift=0.0, max_iter=100, tolerance=1e-8,
                           cg_steps=10, cg_tol=1e-9,
                           ordering=abi.ORDER_MATCH_PREVIOUS,
                           precision=abi.FP64):
    """Reference signature (include/solver.hpp:43-47) on a device H."""
    p = abi.GcgParams(max_iter=max_iter, tol=tolerance, cg_steps=cg_steps,
                      cg_tol=cg_tol, shift=shift, ordering=ordering,
                      precision=precision, precond=0)
    X, lam, _ = H.gcg(X_initial, nev, ConjDir, p)
    return X, lam


def solve(H: Hamiltonian, ConjDir, calc: dict, guess, nev=None,
          precision=abi.FP64):
    """Utilities::solve (src/util/utilities.cpp:20-36): GCG with shift 0 and
    ascending ordering, parameters from a GCGParameters-like dict."""
    nev = guess.shape[1] if nev is None else nev
    return gcgm_complex_no_B_lock(H, guess, ConjDir, nev, 0.0,
                                  calc["maxIter"], calc["tol"], calc["steps"],
                                  calc["cgTol"], abi.ORDER_ASCENDING,
                                  precision)


class IterationData:
    """The self-consistent state of one run (IterationData,
    include/util/iteration_data.hpp:81-137) for a caller that drives its own
    HF loop around the GCG, as main() does (src/main.cpp:199-342):

        data = IterationData(cfg)
        data.update_quantities((Xn, en), (Xp, ep), it)   # densities, fields
        H_n.set_fields(*data.fields(NEUTRON)[:4]); ...      # Hamiltonians
        ... solve ...
        E_int, E_HF = data.energies(new_en, new_ep)
    """

    def __init__(self, cfg: abi.HFConfig):
        self.cfg = cfg
        self.n = cfg.n
        h = C.c_void_p()
        _check(load().ncgm_state_create(C.byref(h), C.byref(cfg)))
        self.h = h

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            load().ncgm_state_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update_quantities(self, neutrons, protons, it,
                          flags=abi.UPDATE_NORMALIZE | abi.UPDATE_TRORDER):
        """IterationData::updateQuantities (iteration_data.cpp:852-1125);
        neutrons / protons: (X, eigenvalues), X in the Eigen layout."""
        (Xn, en), (Xp, ep) = neutrons, protons
        Xn = np.asfortranarray(Xn, dtype=np.complex128)
        Xp = np.asfortranarray(Xp, dtype=np.complex128)
        en = np.ascontiguousarray(en, dtype=np.float64)
        ep = np.ascontiguousarray(ep, dtype=np.float64)
        _check(load().ncgm_state_update(self.h, Xn.ctypes.data, en.ctypes.data,
                                        Xn.shape[1], Xp.ctypes.data,
                                        ep.ctypes.data, Xp.shape[1], int(it),
                                        int(flags)))

    def fields(self, species):
        """(f, grad f, U, W, UC) in the layout of Hamiltonian.set_fields
        (UC is None for neutrons)."""
        ns = self.n ** 3
        f, U, UC = np.zeros(ns), np.zeros(ns), np.zeros(ns)
        gf, W = np.zeros(3 * ns), np.zeros(3 * ns)
        _check(load().ncgm_state_fields(self.h, species, f.ctypes.data,
                                        gf.ctypes.data, U.ctypes.data,
                                        W.ctypes.data, UC.ctypes.data))
        return f, gf, U, W, (UC if species == abi.PROTON else None)

    def densities(self, species):
        """(rho, tau) of a species."""
        ns = self.n ** 3
        rho, tau = np.zeros(ns), np.zeros(ns)
        _check(load().ncgm_state_densities(self.h, species, rho.ctypes.data,
                                           tau.ctypes.data))
        return rho, tau

    def energies(self, en, ep):
        """(E_int, E_HF) of the current densities with the new levels."""
        en = np.ascontiguousarray(en, dtype=np.float64)
        ep = np.ascontiguousarray(ep, dtype=np.float64)
        a, b = C.c_double(), C.c_double()
        _check(load().ncgm_state_energy(self.h, en.ctypes.data, ep.ctypes.data,
                                        C.byref(a), C.byref(b)))
        return a.value, b.value


def hf_run(cfg: abi.HFConfig, outputs: bool = False):
    """Runs the WS guess and HF(B) iteration on the GPU (ncgm_hf_run).
    With outputs, also what the reference's output step reads
    (ncgm_hf_run_ex): the final orbitals, the recomputed kinetic densities,
    the Lagrange-mesh gradients of rho, the mean fields and the energy
    table."""
    res = abi.HFResult()
    on, op = config.orbital_counts(cfg)
    ns = cfg.n ** 3
    spe_n, spe_p = np.zeros(on), np.zeros(op)
    rho_n, rho_p = np.zeros(ns), np.zeros(ns)
    en = np.zeros((max(cfg.max_iterations, 1), 2))
    arrays = {"spe_n": spe_n, "spe_p": spe_p, "rho_n": rho_n, "rho_p": rho_p}
    if not outputs:
        _check(load().ncgm_hf_run(C.byref(cfg), C.byref(res),
                                  spe_n.ctypes.data, spe_p.ctypes.data,
                                  rho_n.ctypes.data, rho_p.ctypes.data,
                                  en.ctypes.data))
    else:
        N = 2 * ns
        extra = {"orbitals_n": np.zeros((N, on), np.complex128, order="F"),
                 "orbitals_p": np.zeros((N, op), np.complex128, order="F"),
                 "tau_n": np.zeros(ns), "tau_p": np.zeros(ns),
                 "grad_rho_n": np.zeros(3 * ns), "grad_rho_p": np.zeros(3 * ns),
                 "U_n": np.zeros(ns), "U_p": np.zeros(ns)}
        out = abi.HFOutputs(**{k: v.ctypes.data for k, v in extra.items()})
        _check(load().ncgm_hf_run_ex(C.byref(cfg), C.byref(res),
                                     spe_n.ctypes.data, spe_p.ctypes.data,
                                     rho_n.ctypes.data, rho_p.ctypes.data,
                                     en.ctypes.data, C.byref(out)))
        for q in ("n", "p"):
            extra["grad_rho_" + q] = extra["grad_rho_" + q].reshape(3, ns).T
        arrays.update(extra)
        arrays["terms"] = np.array(out.terms[:])
        arrays["constraints_energy"] = out.constraints_energy
    arrays["energies"] = en[:res.iterations]
    return res, arrays


def shell_observables(ctx: "Context", psi):
    """ncgm_shell_observables: per column [<L^2>, <J^2>, <Jz Jz>, parity
    overlap, <L.S>] (see include/ncgm.h), shape (ncols, 5)."""
    psi = np.asfortranarray(psi, dtype=np.complex128)
    if psi.ndim == 1:
        psi = psi.reshape(-1, 1, order="F")
    obs = np.zeros((psi.shape[1], 5))
    _check(load().ncgm_shell_observables(ctx.h, psi.ctypes.data, psi.shape[1],
                                         obs.ctypes.data))
    return obs


class LearnedPreconditioner:
    """The GCG correction network (ncgm_lp_*): a 4-level 3-D convolutional
    U-Net with BF16 weights that maps one real component of a GCG residual,
    with the local fields, to a start d0 for the correction PCG. Trained on
    the device on residual / exact-correction pairs that the solver itself
    produces. The reference has no counterpart (its PCG starts from 0)."""

    def __init__(self, seed: int = 1):
        h = C.c_void_p()
        _check(load().ncgm_lp_create(C.byref(h), int(seed)))
        self.h = h
        self.P = load().ncgm_lp_num_params()

    def close(self):
        if self.h:
            load().ncgm_lp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        th = np.zeros(self.P, np.float32)
        _check(load().ncgm_lp_get_params(self.h, th.ctypes.data))
        return th

    @params.setter
    def params(self, th):
        th = np.ascontiguousarray(th, np.float32)
        _check(load().ncgm_lp_set_params(self.h, th.ctypes.data))

    def forward(self, x):
        """x [B, 3, n, n, n] float32 -> y [B, 1, n, n, n]."""
        x = np.ascontiguousarray(x, np.float32)
        B, n = x.shape[0], x.shape[-1]
        y = np.zeros((B, 1, n, n, n), np.float32)
        _check(load().ncgm_lp_forward(self.h, n, B, x.ctypes.data,
                                      y.ctypes.data))
        return y

    def gradient(self, x, t):
        """(loss, dloss/dtheta) for inputs x [B, 3, n^3] and targets t."""
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        B, n = x.shape[0], x.shape[-1]
        g = np.zeros(self.P, np.float32)
        loss = C.c_float()
        _check(load().ncgm_lp_gradient(self.h, n, B, x.ctypes.data,
                                       t.ctypes.data, C.byref(loss),
                                       g.ctypes.data))
        return float(loss.value), g

    def collect(self, H: "Hamiltonian", X, lam, shift, cg_steps=2000,
                cg_tol=1e-10):
        """Adds 4 ncols pairs (r = X lam - H X, exact d of (H + shift) d = r)."""
        X = np.asfortranarray(X, np.complex128)
        lam = np.ascontiguousarray(lam, np.float64)
        _check(load().ncgm_lp_collect(self.h, H.ctx.h, H.species,
                                      X.ctypes.data, X.shape[1],
                                      lam.ctypes.data, float(shift),
                                      int(cg_steps), float(cg_tol)))

    def dataset_size(self, n):
        return load().ncgm_lp_dataset_size(self.h, int(n))

    def train(self, steps, batch=16, lr=1e-3, seed=1):
        curve = np.zeros(steps, np.float32)
        _check(load().ncgm_lp_train(self.h, int(steps), int(batch), float(lr),
                                    int(seed), curve.ctypes.data))
        return curve

    def eval(self, n):
        out = C.c_double()
        _check(load().ncgm_lp_eval(self.h, int(n), C.byref(out)))
        return out.value

    def bind(self, ctx: Context):
        """Network used by ncgm_gcg on ctx with precond = LEARNED."""
        _check(load().ncgm_set_lp(ctx.h, self.h))

    def save(self, path):
        self.params.astype(np.float32).tofile(path)

    @classmethod
    def pretrained(cls, path=None):
        """The network trained by nuclearcgm_gb300.train_lp (data/)."""
        path = path or os.path.join(HERE, "data", "lp_weights.f32")
        lp = cls()
        lp.params = np.fromfile(path, np.float32)
        return lp


def hf_run_batch(cfgs, max_concurrent: int = 0, densities: bool = False):
    """Independent HF runs (e.g. the points of a deformation curve) on one
    GPU, each on its own host thread, context and stream
    (ncgm_hf_run_batch). Returns the list of results and, with
    densities=True, the lists of neutron and proton densities."""
    count = len(cfgs)
    arr = (abi.HFConfig * count)(*cfgs)
    res = (abi.HFResult * count)()
    status = np.zeros(count, np.int32)
    rn = rp = None
    pn = pp = None
    if densities:
        rn = [np.zeros(c.n ** 3) for c in cfgs]
        rp = [np.zeros(c.n ** 3) for c in cfgs]
        pn = (C.c_void_p * count)(*[r.ctypes.data for r in rn])
        pp = (C.c_void_p * count)(*[r.ctypes.data for r in rp])
    _check(load().ncgm_hf_run_batch(arr, count, int(max_concurrent), res,
                                    status.ctypes.data, pn, pp))
    out = list(res)
    return (out, rn, rp) if densities else out
