"""Batched constraint points: the runs of a quadrupole-constrained
deformation curve executed together on one GPU (ncgm_hf_run_batch) give
exactly the results of the same runs one at a time, and each point agrees
with its own FP64 oracle run."""
import time

import numpy as np
import pytest

import nuclearcgm_gb300 as ng
from nuclearcgm_gb300 import config
from oracle import oracle

pytestmark = pytest.mark.gpu

MG24 = {"functional": "SKMstar", "nucleus": {"A": 24, "Z": 12},
        "box": {"boxSize": 16.5, "axisMeshPoints": 12},
        "maxIterations": 60, "energyTol": 1e-6}


def _curve(betas, data=MG24):
    cfgs = []
    for beta, mu in config.curve_points(24, betas[0], betas[-1], len(betas)):
        c = config.from_input(data)
        c.curve_mode = 1
        c.mu20 = mu
        c.initial_beta = beta
        cfgs.append(c)
    return cfgs


def test_batch_equals_sequential_runs():
    cfgs = _curve([-0.3, -0.1, 0.1, 0.3, 0.5])
    t0 = time.perf_counter()
    seq = [ng.hf_run(c) for c in cfgs]
    t_seq = time.perf_counter() - t0
    t0 = time.perf_counter()
    res, rn, rp = ng.hf_run_batch(cfgs, densities=True)
    t_bat = time.perf_counter() - t0
    print("5 curve points: sequential %.2f s, batched %.2f s" % (t_seq,
                                                                  t_bat))
    for (r1, o1), r2, n2, p2 in zip(seq, res, rn, rp):
        assert r2.iterations == r1.iterations
        assert r2.E_HF == r1.E_HF and r2.E_int == r1.E_int
        assert np.array_equal(n2, o1["rho_n"])
        assert np.array_equal(p2, o1["rho_p"])


O16 = {"functional": "SKMstar", "nucleus": {"A": 16, "Z": 8},
       "box": {"boxSize": 16.5, "axisMeshPoints": 12},
       "maxIterations": 300, "energyTol": 1e-7}


def test_batch_points_match_oracle():
    """Constrained points that converge on this small lattice (the oblate
    24Mg points of the batch test oscillate without pairing, and the
    reference's augmented Lagrangian diverges at beta = 0.3 on a 12^3
    lattice, in the oracle as well)."""
    cfgs = []
    for beta, mu in config.curve_points(16, 0.05, 0.15, 2):
        c = config.from_input(O16)
        c.curve_mode = 1
        c.mu20 = mu
        c.initial_beta = beta
        c.hf_gcg.cg_tol = 1e-8
        cfgs.append(c)
    res = ng.hf_run_batch(cfgs, max_concurrent=2)
    for c, r in zip(cfgs, res):
        ro, _ = oracle.hf_run(c)
        print("beta %.3f: E_HF %.6f / %.6f, beta2 %.5f / %.5f" % (
            r.beta, r.E_HF, ro.E_HF, r.beta, ro.beta))
        assert abs(r.E_int - ro.E_int) < 1e-3
        assert abs(r.E_HF - ro.E_HF) < 1e-3
        assert abs(r.beta - ro.beta) < 1e-4
