"""CPU checks of the stored oracle fixed points (tests/golden): each is a
converged fixed point of its configuration (energy settled, densities
normalised to the particle numbers, levels ascending), and the stored input
rebuilds the configuration it was made from."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_fixtures as mf  # noqa: E402


def _weights(n, box):
    h = box / (n - 1)
    w = np.ones(n)
    w[0] = w[-1] = 0.5
    return (w[:, None, None] * w[None, :, None] * w[None, None, :]).ravel() \
        * h ** 3


@pytest.mark.parametrize("name", sorted(mf.CASES))
def test_fixture_is_a_converged_fixed_point(name):
    if not os.path.exists(mf.path(name)):
        pytest.skip("fixture not generated")
    fx = mf.load(name)
    inp, iters, cg_tol, point = mf.CASES[name]
    assert fx["input"] == inp
    assert int(fx["iterations"]) == iters and float(fx["cg_tol"]) == cg_tol
    assert int(fx["curve_point"]) == (-1 if point is None else point)
    en = fx["energies"]
    assert en.shape == (iters, 2)
    # the energy has settled far below the 1 keV comparison tolerance
    assert np.abs(np.diff(en[-20:, 0])).max() < 1e-7
    n = inp["box"]["axisMeshPoints"]
    wt = _weights(n, inp["box"]["boxSize"])
    A, Z = inp["nucleus"]["A"], inp["nucleus"]["Z"]
    assert abs((fx["rho_n"] * wt).sum() - (A - Z)) < 1e-5
    assert abs((fx["rho_p"] * wt).sum() - Z) < 1e-5
    for q in ("spe_n", "spe_p"):
        assert np.all(np.diff(fx[q]) >= -1e-9)
    assert fx["rho_n"].dtype == np.float32 and fx["rho_n"].size == n ** 3
    assert float(fx["E_int"]) == pytest.approx(en[-1, 0], abs=1e-12)


def test_curve_configs_follow_mu20_from_beta():
    from nuclearcgm_gb300 import config
    cfgs = mf.curve_configs(mf.MG24)
    assert len(cfgs) == 16
    pts = config.curve_points(24, -0.3, 0.5, 16)
    for c, (b, mu) in zip(cfgs, pts):
        assert c.curve_mode == 1 and c.mu20 == mu and c.initial_beta == b
    c = mf.make_config(mf.MG24, 400, 1e-8, 7)
    assert c.mu20 == pts[7][1] and c.energy_tol == 0.0
    assert c.max_iterations == 400 and c.hf_gcg.cg_tol == 1e-8
