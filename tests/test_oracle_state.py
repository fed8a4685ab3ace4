"""The oracle's state-update restatement (test infrastructure for the device
state handle): densities of normalised orbitals integrate to the particle
number, and a second update from the same orbitals leaves the mixed
densities unchanged (mixing identical densities is the identity)."""
import numpy as np

from nuclearcgm_gb300 import config
from oracle import oracle

from test_gpu_state import _orbitals


def test_state_run_particle_numbers_and_mixing():
    n, box = 10, 14.0
    data = {"functional": "SLy4", "nucleus": {"A": 16, "Z": 8},
            "box": {"boxSize": box, "axisMeshPoints": n},
            "maxIterations": 1, "energyTol": 0.0}
    cfg = config.from_input(data)
    Xn = _orbitals(n, box, 8, 1)
    Xp = _orbitals(n, box, 8, 2)
    en = np.linspace(-40.0, -5.0, 8)
    ep = np.linspace(-35.0, -2.0, 8)
    r1 = oracle.state_run(cfg, (Xn, en), (Xp, ep), 1, 1)
    r2 = oracle.state_run(cfg, (Xn, en), (Xp, ep), 2, 1)
    h = box / (n - 1)
    w = np.ones(n)
    w[0] = w[-1] = 0.5
    wt = (w[:, None, None] * w[None, :, None] * w[None, None, :]).ravel()
    assert abs((r1["rho_n"] * wt).sum() * h ** 3 - 8.0) < 1e-9
    assert abs((r1["rho_p"] * wt).sum() * h ** 3 - 8.0) < 1e-9
    for k in ("rho_n", "rho_p", "tau_n", "f_n", "W_p"):
        assert np.abs(r1[k] - r2[k]).max() <= 1e-13 * np.abs(r1[k]).max()
    assert np.isfinite(r1["E_int"]) and np.isfinite(r1["E_HF"])
