"""Small, fixed workloads for profiling single kernels of the library
(the commands in profiles/*.md run these).

  python -m nuclearcgm_gb300.profile_cases tcgram      # ncgm_gram, 128 000 x 96
  python -m nuclearcgm_gb300.profile_cases tcprod      # 40Ca shape: A^H A, V C
  python -m nuclearcgm_gb300.profile_cases hf_o16      # 4 HF iterations, 16O 30^3
  python -m nuclearcgm_gb300.profile_cases hf_ca40_tc  # 6 HF iterations, 40Ca 36^3
  python -m nuclearcgm_gb300.profile_cases gcg_step64  # one GCG step, 40^3 x 64
"""
import sys

import numpy as np

from . import Context, Grid, Hamiltonian, _check, abi, config, hf_run, load
from . import workloads


def tcgram():
    """C = A^H A for an orthonormal 2*40^3 x 96 block: FP64, then the
    TF32-split and the exact-digit tensor-core forms."""
    n, p = 40, 96
    ctx = Context(Grid(n, 9.75), 4)
    A = workloads.orthonormal_block(2 * n ** 3, p, seed=5)
    C = np.zeros((p, p), np.complex128, order="F")
    for prec in (abi.FP64, abi.FP32, abi.FP32_TC):
        _check(load().ncgm_gram(ctx.h, A.ctypes.data, p, A.ctypes.data, p,
                                C.ctypes.data, prec))
    print("max |A^H A - I| = %.2e" % np.abs(C - np.eye(p)).max())
    ctx.close()


def tcprod():
    """The exact-digit products at the 40Ca tensor-core run's shape
    (2*36^3 = 93 312 rows, 60 columns): the self-Gram A^H A, then Y = A C
    with C 60 x 20."""
    n, p, k = 36, 60, 20
    N = 2 * n ** 3
    ctx = Context(Grid(n, 10.5), 4)
    A = workloads.orthonormal_block(N, p, seed=1)
    Cm = np.asfortranarray(np.random.default_rng(2).normal(size=(p, k))
                           + 0j)
    G = np.zeros((p, p), np.complex128, order="F")
    Y = np.zeros((N, k), np.complex128, order="F")
    _check(load().ncgm_gram(ctx.h, A.ctypes.data, p, A.ctypes.data, p,
                            G.ctypes.data, abi.FP32_TC))
    _check(load().ncgm_vc(ctx.h, A.ctypes.data, p, Cm.ctypes.data, k,
                          Y.ctypes.data, abi.FP32_TC))
    ref = A @ Cm
    print("max |A^H A - I| = %.2e, max |Y - A C| / max |A C| = %.2e" % (
        np.abs(G - np.eye(p)).max(), np.abs(Y - ref).max() / np.abs(ref).max()))
    ctx.close()


def hf_o16(precision=abi.FP64, iterations=4):
    """HF iterations of 16O (SLy4, box 18 fm, 30^3), four by default."""
    data = {"functional": "SLy4", "nucleus": {"A": 16, "Z": 8},
            "box": {"boxSize": 18.0, "axisMeshPoints": 30},
            "maxIterations": iterations, "energyTol": 0.0}
    res, _ = hf_run(config.from_input(data, precision=precision))
    print("iterations %d wall %.3f s (gcg %.3f, poisson %.3f)" % (
        res.iterations, res.wall_s, res.t_gcg_s, res.t_poisson_s))


def hf_ca40_tc(precision=abi.FP32_TC, iterations=6):
    """Six HF iterations of 40Ca (SLy4, box 20 fm, 36^3) in the mixed
    tensor-core form."""
    data = {"functional": "SLy4", "nucleus": {"A": 40, "Z": 20},
            "box": {"boxSize": 20.0, "axisMeshPoints": 36},
            "maxIterations": iterations, "energyTol": 0.0}
    res, _ = hf_run(config.from_input(data, precision=precision))
    print("iterations %d wall %.3f s (gcg %.3f, poisson %.3f)" % (
        res.iterations, res.wall_s, res.t_gcg_s, res.t_poisson_s))


def gcg_step64(precision=abi.FP64):
    """One GCG iteration on the 40^3 x 64 benchmark workload."""
    a, f, gradf, U, W = workloads.fields(40, 0.5)
    ctx = Context(Grid(40, a), 64)
    H = Hamiltonian(ctx, abi.NEUTRON).set_fields(f, gradf.T, U, W.T)
    X = workloads.orthonormal_block(2 * 40 ** 3, 64, seed=1)
    p = abi.GcgParams(max_iter=1, tol=1e-6, cg_steps=80, cg_tol=1e-5,
                      shift=0, ordering=1, precision=precision, precond=0)
    _, _, st = H.gcg(X, 64, None, p)
    print("GCG step %.1f ms (PCG %.1f ms)" % (st.ms_total, st.ms_pcg))
    ctx.close()


def hf_o16_tc(iterations=4):
    """HF iterations of 16O in the mixed tensor-core form."""
    hf_o16(abi.FP32_TC, iterations)


CASES = {"tcgram": tcgram, "tcprod": tcprod, "hf_o16": hf_o16, "hf_o16_tc": hf_o16_tc,
         "hf_ca40_tc": hf_ca40_tc, "gcg_step64": gcg_step64}

if __name__ == "__main__":
    # optional second argument: the HF iteration count of the hf_* cases
    name = sys.argv[1] if len(sys.argv) > 1 else "tcgram"
    if len(sys.argv) > 2:
        CASES[name](iterations=int(sys.argv[2]))
    else:
        CASES[name]()
