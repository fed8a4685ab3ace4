"""GPU parity of the H.X stencil against the oracle's assembled CSR."""
import numpy as np
import pytest

import nuclearcgm_gb300 as ng
from conftest import random_block, random_fields
from nuclearcgm_gb300 import abi, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12   # max-abs error / max|Y|, FP64 stencil vs CSR
FP32_TOL = 3e-6    # same, FP32 stencil (inputs rounded to FP32)


def _pair(n, a, seed, so=True, coul=False, ncols=3):
    f, gradf, U, W, UC = random_fields(n, seed, so=so, coulomb=coul)
    ctx = ng.Context(ng.Grid(n, a), max_cols=max(ncols, 4))
    H = ng.Hamiltonian(ctx, abi.PROTON).set_fields(f, gradf, U, W, UC)
    R = oracle.Hamiltonian.skyrme(n, a, f, gradf, U, W, UC)
    return ctx, H, R


@pytest.mark.parametrize("n,so,coul", [(6, True, False), (9, True, True),
                                       (12, False, True), (16, True, True),
                                       (21, True, False)])
def test_fp64_matches_csr(n, so, coul):
    a = 0.5 * (n - 1) * 0.7
    ctx, H, R = _pair(n, a, 100 + n, so, coul)
    X = random_block(2 * n ** 3, 3, n)
    Y, ref = H.apply(X), R.apply(X)
    assert np.abs(Y - ref).max() <= FP64_TOL * np.abs(ref).max()


@pytest.mark.parametrize("n", [6, 13, 24, 40])
def test_fp32_plane_kernel_error_bound(n):
    a = 0.5 * (n - 1) * 0.5
    ctx, H, R = _pair(n, a, 7 + n, True, True, ncols=5)
    X = random_block(2 * n ** 3, 5, 2 * n)
    Y32 = H.apply(X, abi.FP32)
    ref = R.apply(X)
    assert np.abs(Y32 - ref).max() <= FP32_TOL * np.abs(ref).max()


# fixed stencil shapes (rows, ring, ppt, CTAs/SM, kind, cpa, nc), bypassing
# the autotuner: kind 0 = plane-streaming kernel (cpa: coefficient
# prefetch), kind 1 = z-marching kernel, kind 2 = staged-coefficient kernel
# (ppt: rows per thread, cpa: coefficient ring depth, nc: columns per box),
# kind 3 = kind 2 with the z-neighbours in registers
SHAPES = ["3,8,1,1,0", "5,16,4,2,0", "10,8,2,1,0,1", "5,16,4,2,0,1",
          "2,4,1,1,1", "8,8,1,2,1", "12,8,1,1,1", "6,4,1,4,1",
          "12,8,2,1,2,2,1", "10,8,1,1,2,4,2", "8,8,4,1,2,2,1",
          "6,8,2,1,2,4,2", "4,8,4,2,2,2,1", "2,8,1,1,2,2,2",
          "12,8,2,1,3,2,1", "8,8,2,2,3,2,1", "8,16,4,1,3,4,1",
          "6,8,1,2,3,8,1", "2,8,1,1,3,2,1"]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("n", [12, 40])
def test_fp32_fixed_shapes(monkeypatch, shape, n):
    """Every kernel form and pipeline depth gives the CSR product (the
    shape is read when a context tunes; shapes invalid for a lattice fall
    back to the tuner). Five columns: the two-column boxes end on a
    half-empty box."""
    monkeypatch.setenv("NCGM_STENCIL_SHAPE", shape)
    a = 0.5 * (n - 1) * 0.5
    ctx, H, R = _pair(n, a, 300 + n, True, True, ncols=6)
    X = random_block(2 * n ** 3, 5, 3 * n)
    Y32 = H.apply(X, abi.FP32)
    ref = R.apply(X)
    assert np.abs(Y32 - ref).max() <= FP32_TOL * np.abs(ref).max()
    ctx.close()


def test_device_and_host_pointers_agree():
    torch = pytest.importorskip("torch")
    n, a = 10, 3.0
    ctx, H, R = _pair(n, a, 3)
    X = random_block(2 * n ** 3, 2, 1)
    Yh = H.apply(X)
    Xd = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()  # col-major data
    Yd = H.apply(Xd).cpu().numpy().T
    assert np.array_equal(Yh, Yd)


def test_woods_saxon_fields_on_device():
    n, a, A, Z = 12, 5.5, 24, 12
    ctx = ng.Context(ng.Grid(n, a), 4)
    H = ng.Hamiltonian(ctx, abi.NEUTRON).set_woods_saxon(A, Z, beta=0.2)
    R = oracle.Hamiltonian.woods_saxon(n, a, A, Z, beta=0.2)
    X = random_block(2 * n ** 3, 2, 5)
    Y, ref = H.apply(X), R.apply(X)
    assert np.abs(Y - ref).max() <= 1e-11 * np.abs(ref).max()


def test_bad_arguments_return_status():
    n, a = 8, 3.0
    ctx = ng.Context(ng.Grid(n, a), 2)
    H = ng.Hamiltonian(ctx, abi.NEUTRON)
    X = random_block(2 * n ** 3, 1, 0)
    with pytest.raises(ng.NcgmError) as e:
        H.apply(X)  # fields not set
    assert e.value.status == abi.NCGM_OK + 1
    f, gradf, U, W, UC = random_fields(n, 1)
    H.set_fields(f, gradf, U, W)
    with pytest.raises(ng.NcgmError):
        H.apply(random_block(2 * n ** 3, 3, 0))  # more than max_cols
    with pytest.raises(ng.NcgmError):
        ng.Hamiltonian(ctx, 2).set_fields(f, gradf, U, W)


def test_full_size_linearity_and_fp32_error():
    """40^3 lattice, 64 spinors (the benchmark workload): FP64 linearity
    H(aX + bZ) = aHX + bHZ and the FP32 error against FP64."""
    a, f, gradf, U, W = workloads.fields(40, 0.5)
    ctx = ng.Context(ng.Grid(40, a), 64)
    H = ng.Hamiltonian(ctx, abi.NEUTRON).set_fields(f, gradf.T, U, W.T)
    X = workloads.orthonormal_block(2 * 40 ** 3, 64, seed=1)
    Z = np.asfortranarray(np.roll(X, 1, axis=1))
    al, be = 0.3 - 0.2j, -1.1 + 0.4j
    Y = H.apply(al * X + be * Z)
    Yl = al * H.apply(X) + be * H.apply(Z)
    assert np.abs(Y - Yl).max() <= 1e-12 * np.abs(Y).max()
    Y64 = H.apply(X)
    Y32 = H.apply(X, abi.FP32)
    assert np.abs(Y32 - Y64).max() <= FP32_TOL * np.abs(Y64).max()


@pytest.mark.parametrize("precision", [abi.FP64, abi.FP32])
def test_host_pipeline_matches_device_apply(precision):
    """Host buffers with more columns than one ~16 MB chunk (40^3: 8 columns
    per chunk) take the chunked copy-in / apply / copy-out pipeline; every
    column must equal the single device-side apply bit for bit (20 columns:
    chunks of 8, 8 and 4)."""
    torch = pytest.importorskip("torch")
    a, f, gradf, U, W = workloads.fields(40, 0.5)
    ctx = ng.Context(ng.Grid(40, a), 20)
    H = ng.Hamiltonian(ctx, abi.NEUTRON).set_fields(f, gradf.T, U, W.T)
    X = workloads.orthonormal_block(2 * 40 ** 3, 20, seed=4)
    Yh = H.apply(X, precision)
    if precision == abi.FP64:
        Xd = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
        Yd = H.apply(Xd).cpu().numpy().T
    else:
        Xd = torch.from_numpy(np.ascontiguousarray(X.T)).to(torch.complex64).cuda()
        Yd = torch.empty_like(Xd)
        ng._check(ng.load().ncgm_apply_h_device(ctx.h, abi.NEUTRON, Xd.data_ptr(),
                                                Yd.data_ptr(), 20, abi.FP32,
                                                0.0))
        torch.cuda.synchronize()
        Yd = Yd.cpu().numpy().T.astype(np.complex128)
    assert np.array_equal(Yh, Yd)
    ctx.close()
