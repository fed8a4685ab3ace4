"""The IterationData-shaped state handle (ncgm_state_*, replacing
IterationData::updateQuantities, src/util/iteration_data.cpp:852-1125) and,
through it, the density, mean-field, mixing and Coulomb kernels, checked
directly against the oracle's restatement of the same update on smooth
random orbitals (not only through a converged fixed point):

  * f = hbar^2/2m*, grad f, U (central + constraint), W (spin-orbit) and the
    densities rho, tau to 1e-12 relative (max |d| / max |value|);
  * the Coulomb field to 1e-9 relative (both sides stop their Poisson
    solves at a 1e-13 relative residual, with different solvers);
  * E_int and E_HF with new levels to 1e-7 MeV.

Two updates are made in a row, so the second exercises the density mixing
(iteration 1 mixes with the first update's densities)."""
import numpy as np
import pytest

import nuclearcgm_gb300 as ng
from nuclearcgm_gb300 import abi, config
from oracle import oracle

pytestmark = pytest.mark.gpu

N_LAT, BOX = 16, 16.0


def _orbitals(n, box, ncols, seed, tr_pairs=False):
    """Smooth random 2-spinors: each component a sum of three Gaussians
    with random centres, widths and complex weights (Eigen layout, rows
    s + 2(i + n(j + n k))). With tr_pairs, column 2k+1 is i sigma_y times
    the conjugate of column 2k."""
    rng = np.random.default_rng(seed)
    a = box / 2
    x = -a + np.arange(n) * box / (n - 1)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")  # [k][j][i]
    out = np.zeros((2 * n ** 3, ncols), np.complex128)
    for c in range(ncols):
        if tr_pairs and c % 2 == 1:
            up, dn = out[0::2, c - 1], out[1::2, c - 1]
            out[0::2, c] = np.conj(dn)
            out[1::2, c] = -np.conj(up)
            continue
        for s in range(2):
            v = np.zeros_like(X, dtype=np.complex128)
            for _ in range(3):
                c0 = rng.uniform(-2.5, 2.5, 3)
                w = rng.uniform(1.5, 2.5)
                amp = rng.normal() + 1j * rng.normal()
                v += amp * np.exp(-((X - c0[0]) ** 2 + (Y - c0[1]) ** 2 +
                                    (Z - c0[2]) ** 2) / (2 * w * w))
            out[s::2, c] = v.reshape(-1)
    return out


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _check(cfg, neutrons, protons, flags):
    rng = np.random.default_rng(5)
    en2 = np.sort(neutrons[1] + rng.normal(0, 0.1, len(neutrons[1])))
    ep2 = np.sort(protons[1] + rng.normal(0, 0.1, len(protons[1])))
    data = ng.IterationData(cfg)
    for it in range(2):
        data.update_quantities(neutrons, protons, it, flags)
    E_int, E_HF = data.energies(en2, ep2)
    ref = oracle.state_run(cfg, neutrons, protons, 2, flags, (en2, ep2))
    worst = {}
    for q, sp in (("n", abi.NEUTRON), ("p", abi.PROTON)):
        f, gf, U, W, UC = data.fields(sp)
        rho, tau = data.densities(sp)
        for name, v in (("f", f), ("gradf", gf), ("U", U), ("W", W),
                        ("rho", rho), ("tau", tau)):
            worst[name + "_" + q] = _rel(v, ref[name + "_" + q])
        if UC is not None and np.abs(ref["UC_p"]).max() > 0:
            worst["UC_p"] = _rel(UC, ref["UC_p"])
    print({k: "%.1e" % v for k, v in worst.items()},
          "E_int %.9f / %.9f, E_HF %.9f / %.9f" % (E_int, ref["E_int"], E_HF,
                                                   ref["E_HF"]))
    for k, v in worst.items():
        assert v < (1e-9 if k.startswith("UC") else 1e-12), (k, v)
    assert abs(E_int - ref["E_int"]) < 1e-7
    assert abs(E_HF - ref["E_HF"]) < 1e-7
    data.close()


def test_state_update_fields_match_oracle_hf():
    """16O, SLy4, Coulomb, no pairing: 8 + 8 orbitals."""
    data = {"functional": "SLy4", "nucleus": {"A": 16, "Z": 8},
            "box": {"boxSize": BOX, "axisMeshPoints": N_LAT},
            "maxIterations": 1, "energyTol": 0.0}
    cfg = config.from_input(data)
    Xn = _orbitals(N_LAT, BOX, 8, 1)
    Xp = _orbitals(N_LAT, BOX, 8, 2)
    en = np.linspace(-40.0, -5.0, 8)
    ep = np.linspace(-35.0, -2.0, 8)
    _check(cfg, (Xn, en), (Xp, ep), abi.UPDATE_NORMALIZE)


def test_state_update_fields_match_oracle_bcs():
    """24Mg, SkM*, Coulomb, BCS with 16 states per isospin (time-reversal
    pairs), normalised and TR-ordered first as main() does."""
    data = {"functional": "SKMstar", "nucleus": {"A": 24, "Z": 12},
            "box": {"boxSize": BOX, "axisMeshPoints": N_LAT},
            "maxIterations": 1, "energyTol": 0.0,
            "pairing": {"type": "BCS", "HFbasisSize": 16, "V0": 300.0,
                        "window": 5.0}}
    cfg = config.from_input(data)
    Xn = _orbitals(N_LAT, BOX, 16, 3, tr_pairs=True)
    Xp = _orbitals(N_LAT, BOX, 16, 4, tr_pairs=True)
    en = np.repeat(np.linspace(-40.0, -2.0, 8), 2)
    ep = np.repeat(np.linspace(-36.0, 0.5, 8), 2)
    _check(cfg, (Xn, en), (Xp, ep),
           abi.UPDATE_NORMALIZE | abi.UPDATE_TRORDER)


def test_state_rejects_wrong_column_counts():
    data = {"functional": "SLy4", "nucleus": {"A": 16, "Z": 8},
            "box": {"boxSize": BOX, "axisMeshPoints": N_LAT},
            "maxIterations": 1, "energyTol": 0.0}
    st = ng.IterationData(config.from_input(data))
    X = _orbitals(N_LAT, BOX, 6, 1)
    with pytest.raises(RuntimeError):
        st.update_quantities((X, np.zeros(6)), (X, np.zeros(6)), 0)
    st.close()
