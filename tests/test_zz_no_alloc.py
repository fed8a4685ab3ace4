"""The allocation-free Coulomb Poisson entry point, for callers that cannot
allocate device memory (hosts whose framework owns the GPU's memory through
its own pool, or loops that must not stall on cudaMalloc/cudaFree). It must
give the same potential as the allocating ncgm_poisson, call after call,
while its scratch is a static device array shared by all calls.

This file is collected last on purpose: a failure here leaves every other
test already run."""
import ctypes as C

import numpy as np
import pytest

import nuclearcgm_gb300 as ng

pytestmark = pytest.mark.gpu

# The allocating call is pinned to its CG path (NCGM_POISSON_FAST=0): both
# entry points then run the same CG kernels in the same order from U = 0 to
# the same 1e-13 relative residual, so they agree to rounding.
REL_TOL = 1e-12


def _rho(n, a, Z, w, zfac):
    h = 2 * a / (n - 1)
    xs = -a + np.arange(n) * h
    Zg, Yg, Xg = np.meshgrid(xs, xs, xs, indexing="ij")
    rho = np.exp(-(Xg ** 2 + Yg ** 2 + zfac * Zg ** 2) / w ** 2).ravel()
    wt = np.ones((n, n, n))
    for ax in range(3):
        sl = [slice(None)] * 3
        sl[ax] = 0
        wt[tuple(sl)] *= 0.5
        sl[ax] = n - 1
        wt[tuple(sl)] *= 0.5
    return rho * Z / (rho * wt.ravel()).sum() / h ** 3


def test_noalloc_poisson_matches_allocating_call_twice(monkeypatch):
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("NCGM_POISSON_FAST", "0")
    lib = ng.load()
    n, a, Z = 24, 11.0, 20
    ctx = ng.Context(ng.Grid(n, a), 2)
    ns = n ** 3
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row on different densities (the second reuses the
    # scratch the first one left behind)
    for w, zfac in ((2.5, 1.3), (3.0, 0.8)):
        rho = _rho(n, a, Z, w, zfac)
        U_ref, UC_ref = np.zeros(ns), np.zeros(ns)
        ng._check(lib.ncgm_poisson(ctx.h, rho.ctypes.data, Z, None,
                                   U_ref.ctypes.data, UC_ref.ctypes.data,
                                   None))
        d_rho = torch.from_numpy(rho).cuda()
        d_U = torch.empty(ns, dtype=torch.float64, device="cuda")
        d_UC = torch.empty(ns, dtype=torch.float64, device="cuda")
        its = C.c_int(0)
        ng._check(lib.ncgm_poisson_noalloc(n, a, d_rho.data_ptr(), Z, None,
                                           d_U.data_ptr(), d_UC.data_ptr(),
                                           stream, C.byref(its)))
        U, UC = d_U.cpu().numpy(), d_UC.cpu().numpy()
        assert its.value > 0
        assert np.abs(U - U_ref).max() <= REL_TOL * np.abs(U_ref).max()
        assert np.abs(UC - UC_ref).max() <= REL_TOL * np.abs(UC_ref).max()


def test_noalloc_poisson_rejects_oversize_and_host_buffers():
    torch = pytest.importorskip("torch")
    lib = ng.load()
    n = 50  # above NCGM_POISSON_NOALLOC_MAX_N
    d = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
    st = lib.ncgm_poisson_noalloc(n, 10.0, d.data_ptr(), 8, None,
                                  d.data_ptr(), None, None, None)
    assert st == 1 and b"static scratch limit" in lib.ncgm_last_error()
    h = np.zeros(24 ** 3)
    st = lib.ncgm_poisson_noalloc(24, 10.0, h.ctypes.data, 8, None,
                                  h.ctypes.data, None, None, None)
    assert st == 1 and b"device memory" in lib.ncgm_last_error()
