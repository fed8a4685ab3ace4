"""End-to-end parity of the self-consistent iteration (WS guess + HF loop)
between the GPU driver and the FP64 oracle on small lattices.

Two kinds of checks: the iteration trajectory (same number of HF iterations,
energies compared iteration by iteration) and the converged fixed point
against the tolerances of the hot-path target (E 1 keV, single-particle
energies 1e-5 MeV, densities 1e-7 fm^-3)."""
import numpy as np
import pytest

import nuclearcgm_gb300 as ng
from nuclearcgm_gb300 import abi, config
from oracle import oracle

pytestmark = pytest.mark.gpu

E_TOL = 1e-3     # MeV: total energy (1 keV)
SPE_TOL = 1e-5   # MeV: single-particle energies
RHO_TOL = 1e-7   # fm^-3: densities, max-abs

O16 = {"functional": "SLy4", "nucleus": {"A": 16, "Z": 8},
       "box": {"boxSize": 16.5, "axisMeshPoints": 12},
       "maxIterations": 600, "energyTol": 1e-9}


def _run_both(data, precision=abi.FP64, smooth=False, **over):
    cfg = config.from_input(data, precision=precision)
    for k, v in over.items():
        setattr(cfg, k, v)
    if smooth:
        _smooth(cfg)
    res_g, out_g = ng.hf_run(cfg)
    res_o, out_o = oracle.hf_run(cfg)
    return cfg, res_g, out_g, res_o, out_o


def _fixed_point(res_g, out_g, res_o, out_o):
    # both runs are within ~1e-9 MeV per iteration of the fixed point
    assert res_g.last_dE < 1e-8 and res_o.last_dE < 1e-8
    assert abs(res_g.E_int - res_o.E_int) < E_TOL
    assert abs(res_g.E_HF - res_o.E_HF) < E_TOL
    assert np.abs(out_g["spe_n"] - out_o["spe_n"]).max() < SPE_TOL
    assert np.abs(out_g["spe_p"] - out_o["spe_p"]).max() < SPE_TOL
    assert np.abs(out_g["rho_n"] - out_o["rho_n"]).max() < RHO_TOL
    assert np.abs(out_g["rho_p"] - out_o["rho_p"]).max() < RHO_TOL


def _smooth(cfg):
    """Make the iteration a smooth map: every PCG takes all its steps
    (cgTol 0) and the guess solver never locks (tol 0), so no discrete
    decision can fall differently on the two machines."""
    cfg.hf_gcg.cg_tol = 0.0
    cfg.ws_gcg.cg_tol = 0.0
    cfg.ws_gcg.tol = 0.0


def _trajectory(res_g, out_g, res_o, out_o, tol=1e-6):
    assert res_g.iterations == res_o.iterations
    d = np.abs(out_g["energies"] - out_o["energies"]).max()
    assert d < tol, "max energy difference along the iteration %g" % d


def test_o16_hf_fp64_fixed_point():
    _, rg, og, ro, oo = _run_both(O16)
    _fixed_point(rg, og, ro, oo)


def test_o16_hf_fp64_trajectory():
    data = dict(O16, maxIterations=40, energyTol=0.0)
    _, rg, og, ro, oo = _run_both(data, smooth=True)
    _trajectory(rg, og, ro, oo)
    assert np.abs(og["rho_n"] - oo["rho_n"]).max() < 1e-9


def test_o16_hf_mixed_precision_fixed_point():
    """FP32 PCG correction, FP64 Rayleigh-Ritz/residual: same fixed point."""
    _, rg, og, ro, oo = _run_both(O16, precision=abi.FP32)
    _fixed_point(rg, og, ro, oo)


def test_n_equals_z_without_coulomb_copies_neutrons():
    data = {"functional": "SKMstar", "nucleus": {"A": 16, "Z": 8},
            "box": {"boxSize": 16.5, "axisMeshPoints": 12},
            "coulombInteraction": False,
            "maxIterations": 40, "energyTol": 0.0}
    _, rg, og, ro, oo = _run_both(data, smooth=True)
    _trajectory(rg, og, ro, oo)
    assert np.array_equal(og["spe_n"], og["spe_p"])
    assert np.array_equal(og["rho_n"], og["rho_p"])


def test_mg24_bcs_trajectory():
    data = {"functional": "SKMstar", "nucleus": {"A": 24, "Z": 12},
            "box": {"boxSize": 17.0, "axisMeshPoints": 12},
            "pairing": {"type": "BCS", "HFbasisSize": 16, "V0": 1000.0,
                        "window": 5.0},
            "maxIterations": 25, "energyTol": 0.0}
    _, rg, og, ro, oo = _run_both(data, smooth=True)
    _trajectory(rg, og, ro, oo, tol=1e-5)
    assert abs(rg.lambda_n - ro.lambda_n) < 1e-5
    assert abs(rg.E_pair_n - ro.E_pair_n) < 1e-5


def test_quadrupole_constrained_trajectory():
    (beta, mu20), = config.curve_points(24, 0.3, 0.3, 1)
    data = {"functional": "SKMstar", "nucleus": {"A": 24, "Z": 12},
            "box": {"boxSize": 17.0, "axisMeshPoints": 12},
            "maxIterations": 25, "energyTol": 0.0}
    _, rg, og, ro, oo = _run_both(data, smooth=True, curve_mode=1, mu20=mu20,
                                  initial_beta=0.3)
    _trajectory(rg, og, ro, oo, tol=1e-5)
    assert abs(rg.beta - ro.beta) < 1e-6
