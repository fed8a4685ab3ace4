"""The output step's writer (nuclearcgm_gb300.output) on synthetic run
results: file layout, data.json appends, the Eigen matrix text format and
the reference's quirks (pretty(), the swapped counts of the charge
radius). No GPU: the single-particle classification is passed in."""
import json
import math
import os

import numpy as np
import pytest

from nuclearcgm_gb300 import abi, config, output


def _fake(n=6, A=16, Z=8, seed=3):
    rng = np.random.default_rng(seed)
    data = {"functional": "SLy4", "nucleus": {"A": A, "Z": Z},
            "box": {"boxSize": 10.0, "axisMeshPoints": n},
            "maxIterations": 3, "energyTol": 1e-3}
    cfg = config.from_input(data)
    res = abi.HFResult(iterations=3, converged=1, E_int=-120.5, E_HF=-121.0,
                       beta=0.01, gamma=0.2, wall_s=1.5,
                       E_int_lagrange=-119.75)
    ns = n ** 3
    arr = {"rho_n": rng.random(ns) * 0.08, "rho_p": rng.random(ns) * 0.07,
           "tau_n": rng.random(ns), "tau_p": rng.random(ns),
           "U_n": -rng.random(ns) * 50, "U_p": -rng.random(ns) * 40,
           "grad_rho_n": rng.standard_normal((ns, 3)) * 0.01,
           "grad_rho_p": rng.standard_normal((ns, 3)) * 0.01,
           "spe_n": np.sort(rng.random(8) * -30),
           "spe_p": np.sort(rng.random(8) * -25),
           "energies": rng.standard_normal((3, 2)) - 120,
           "terms": np.arange(16, dtype=float), "constraints_energy": 0.25}
    hb2 = output.HBAR ** 2
    obs = np.array([[2 * hb2, 3.75 * hb2, 2.25 * hb2, -1.0, 0.5 * hb2]] * 8)
    shells = (output.classify(obs), output.classify(obs), obs, obs)
    return data, cfg, res, arr, shells


def test_writer_files_and_data_json_appends(tmp_path):
    data, cfg, res, arr, shells = _fake()
    log = ["tot_energies", "hf_energies", "multipoles_2"]
    for _ in range(2):
        output.write(str(tmp_path), "o16", data, cfg, res, arr, shells, log)
    out = tmp_path / "o16_output"
    for f in ("density.csv", "density_n.csv", "density_p.csv",
              "kinetic_n.csv", "kinetic_p.csv", "Field_n.csv", "Field_p.csv",
              "nabla2rho_n.csv", "nabla2rho_p.csv", "C.csv", "C_n.csv",
              "C_p.csv"):
        assert (out / "fields" / f).exists(), f
    doc = json.loads((out / "data" / "data.json").read_text())
    assert len(doc["data"]) == 2
    e = doc["data"][0]
    assert set(e) == {"beta", "betaReal", "EintLag", "Eint", "EpairN",
                      "EpairP", "gamma", "a", "iter", "constraintsEnergy",
                      "step"}
    assert e["EintLag"] == -119.75 and e["Eint"] == -120.5
    assert e["gamma"] == pytest.approx(0.2 * 180 / math.pi)
    assert e["iter"] == 3 and e["constraintsEnergy"] == 0.25
    assert e["step"] == pytest.approx(10.0 / 5)
    en = np.loadtxt(out / "data" / "int_energies.csv")
    assert np.allclose(en, arr["energies"][:, 0], rtol=0, atol=1e-12)
    txt = (tmp_path / "o16_log.txt").read_text()
    assert txt.count("=== Density Functional contributions ===") == 2
    assert "Lagrange recomputed energy: -119.75 MeV" in txt
    assert "C0 Rho0: 1 MeV" in txt and "E coulomb exchange: 14 MeV" in txt
    assert "E (REA): 15 MeV" in txt
    # multipoles_2: l = 0, 1, 2
    assert txt.count("l: ") == 2 * 3
    # the density file re-reads as the n^3 vector
    rho = np.loadtxt(out / "fields" / "density.csv")
    assert np.allclose(rho, arr["rho_n"] + arr["rho_p"], rtol=1e-5)
    g = np.loadtxt(out / "fields" / "nabla2rho_n.csv")
    assert g.shape == (6 ** 3, 3)


def test_eigen_matrix_text_alignment():
    txt = output.matrix_text(np.array([[1.0, -0.5], [1234567.0, 2e-7]]))
    # width 11 (the widest cell), one space between cells
    assert txt.split("\n") == ["          1        -0.5",
                               "1.23457e+06       2e-07"]


def test_reference_quirks():
    # pretty keeps the first character of std::to_string(2x)
    assert output.pretty(1.5) == "3/2"
    assert output.pretty(5.5) == "1/2"
    assert output.round_hi(1.49) == 1.5 and output.round_hi(2.6) == 2.5
    # charge radius: counts swapped (N = Z_in, Z = A - Z_in)
    data, cfg, res, arr, shells = _fake(A=20, Z=8)
    nd = output.nuclear_data(arr, 6, 5.0, 20, 8, shells[2], shells[3])
    corr = (8 * output.MU_N + 8 * output.MU_P) * 0.5
    corr *= 2.0 * (output.HBAR ** 2 / output.MASS ** 2) / 12
    want = abs(nd["rp2"] + 8 * output.RN2 / 12 + output.RP2 + corr)
    assert nd["cr2"] == pytest.approx(want, rel=1e-14)


def test_localisation_bounded():
    rng = np.random.default_rng(1)
    rho = rng.random(50) * 0.1
    tau = rng.random(50)
    g = rng.standard_normal((50, 3)) * 0.01
    C = output.localisation(tau, rho, g)
    assert np.all((C > 0) & (C <= 1))


def test_spherical_harmonics_match_scipy():
    """SphericalHarmonics::Y as the writer restates it equals the standard
    Y_lm with the Condon-Shortley phase (scipy.special.sph_harm_y)."""
    sp = pytest.importorskip("scipy.special")
    if not hasattr(sp, "sph_harm_y"):
        pytest.skip("scipy without sph_harm_y")
    rng = np.random.default_rng(2)
    X, Y, Z = rng.standard_normal((3, 40))
    r = np.sqrt(X * X + Y * Y + Z * Z)
    th, ph = np.arccos(Z / r), np.arctan2(Y, X)
    for l in range(6):
        for m in range(-l, l + 1):
            ref = sp.sph_harm_y(l, m, th, ph)
            assert np.abs(output.ylm(l, m, X, Y, Z) - ref).max() < 1e-13


def test_monopole_is_particle_number_over_sqrt_4pi():
    """Q(0, 0) = int rho Y_00 = A / sqrt(4 pi) for a density normalised to A
    with the trapezoid rule (even n: no lattice point at the origin)."""
    n, a = 12, 6.0
    X, Y, Z, _ = output._coords(n, a)
    rho = np.exp(-(X * X + Y * Y + Z * Z) / 4.0)
    rho *= 16.0 / output.integral(rho, n, a)
    q = output.multipole(0, 0, rho, n, a)
    assert q.real == pytest.approx(16.0 / math.sqrt(4 * math.pi), rel=1e-12)
    assert abs(q.imag) < 1e-12
