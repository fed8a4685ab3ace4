"""The output step of a run: the files the reference's Output::shellsToFile
(src/system/output.cpp:97-408) writes after the HF loop, from the arrays of
hf_run(cfg, outputs=True).

  <folder>/<name>_log.txt                    appended: box, nucleus,
      functional, radii, deformation, convergence, the energy table, HF
      energies, the Lagrange-mesh energy, the single-particle states and
      the multipole moments (when the input's "log" asks for them)
  <folder>/<name>_output/data/data.json      one entry appended per run
      (beta, betaReal, EintLag, Eint, EpairN, EpairP, gamma, a, iter,
      constraintsEnergy, step), the file the plotting scripts read
  <folder>/<name>_output/data/int_energies.csv, hf_energies.csv
      per-iteration energies when "tot_energies" / "hf_energies" are logged
  <folder>/<name>_output/fields/*.csv        density, density_n/p,
      kinetic_n/p, Field_n/p, nabla2rho_n/p (the Lagrange-mesh gradient, as
      the reference writes it under that name) and the localisation
      functions C, C_n, C_p

The quantities of the single-particle table (l, j, mj, parity) come from
ncgm_shell_observables on the GPU; everything else here is arithmetic on
the returned n^3 arrays. Reference quirks kept: the neutron and proton
counts passed to the charge radius are swapped (output.cpp:107-108), the
j / mj strings keep only the first character of 2j (wavefunction.cpp:
519-521), and x^2 moments are plain (unweighted) sums.
"""
import json
import math
import os

import numpy as np

from . import abi

HBAR = 197.327053   # nuclearConstants::h_bar (MeV fm)
MASS = 938.91869    # nuclearConstants::m (MeV)
RP2 = 0.64          # nuclearConstants::rp (fm^2)
RN2 = -0.11         # nuclearConstants::rn (fm^2)
MU_N = -1.913043    # nuclearConstants::muN
MU_P = 2.792847     # nuclearConstants::muP


# --- formatting --------------------------------------------------------------

def fmt(x):
    """A double as std::ostream prints it by default (6 significant
    digits, %g)."""
    return "%g" % x


def matrix_text(m):
    """Eigen's default `stream << matrix`: 6 significant digits, every
    coefficient right-aligned to the widest one, one row per line."""
    m = np.asarray(m, dtype=float)
    if m.ndim == 1:
        m = m.reshape(-1, 1)
    cells = [[fmt(v) for v in row] for row in m]
    w = max((len(c) for row in cells for c in row), default=0)
    return "\n".join(" ".join(c.rjust(w) for c in row) for row in cells)


def write_matrix(path, m):
    with open(path, "w") as f:
        f.write(matrix_text(m) + "\n")


# --- shells (src/util/shell.cpp) ---------------------------------------------

def mom_from_sq(x):
    """momFromSq: l from l(l+1) (shell.cpp:16)."""
    return 0.5 * (-1.0 + math.sqrt(1.0 + 4.0 * x))


def round_hi(x):
    """roundHI (shell.cpp:7-15): to the nearest half-odd integer."""
    c, f = math.ceil(x * 2), math.floor(x * 2)
    return f / 2.0 if c % 2 == 0 else c / 2.0


def pretty(x):
    """pretty (wavefunction.cpp:519-521): first character of
    std::to_string(2x) followed by "/2"."""
    return ("%f" % (x * 2))[:1] + "/2"


def classify(obs):
    """(l, j, mj, parity) per column from ncgm_shell_observables rows
    (Shell::l / j / mj / P, shell.cpp:22-51)."""
    out = []
    h2 = HBAR * HBAR
    for L2, J2, JJ, par, _ in obs:
        l = float(round(mom_from_sq(L2 / h2)))
        j = round_hi(mom_from_sq(J2 / h2))
        mj = round_hi(math.sqrt(JJ) / HBAR) if JJ >= 0 else float("nan")
        out.append((l, j, mj, par))
    return out


def shells_table(shells, energies):
    """The single-particle table (columns l, j, mj, parity, energy_mev)."""
    head = ["l", "j", "mj", "parity", "energy_mev"]
    rows = [[fmt(l), pretty(j), pretty(mj), "+" if p > 0 else "-", fmt(e)]
            for (l, j, mj, p), e in zip(shells, energies)]
    w = [max([len(h)] + [len(r[c]) for r in rows]) for c, h in enumerate(head)]
    line = "-" * (sum(w) + 3 * len(w) + 1)
    txt = [line, "| " + " | ".join(h.ljust(w[c]) for c, h in
                                   enumerate(head)) + " |", line]
    for r in rows:
        txt.append("| " + " | ".join(v.rjust(w[c]) for c, v in
                                     enumerate(r)) + " |")
    txt.append(line)
    return "\n".join(txt)


# --- lattice integrals -------------------------------------------------------

def _coords(n, a):
    xs = -a + np.arange(n) * (2.0 * a / (n - 1))
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    return X.ravel(), Y.ravel(), Z.ravel(), xs


def _trap(n):
    w1 = np.ones(n)
    w1[0] = w1[-1] = 0.5
    return np.einsum("k,j,i->kji", w1, w1, w1).ravel()


def integral(v, n, a):
    """Operators::integral: trapezoid weights times h^3."""
    h = 2.0 * a / (n - 1)
    return float(np.sum(_trap(n) * v) * h ** 3)


def _legendre(l, m, x):
    """associatedLegendre (spherical_harmonics.cpp:14-43), no Condon-Shortley
    sign inside."""
    pmm = np.ones_like(x)
    if m > 0:
        fact = 1.0
        for i in range(1, 2 * m, 2):
            fact *= i
        pmm = fact * np.power(1.0 - x * x, m / 2.0)
    if l == m:
        return pmm
    pmmp1 = x * (2 * m + 1) * pmm
    if l == m + 1:
        return pmmp1
    p1, p2 = pmmp1, pmm
    for ll in range(m + 2, l + 1):
        pll = ((2 * ll - 1) * x * p1 - (ll + m - 1) * p2) / (ll - m)
        p2, p1 = p1, pll
    return p1


def ylm(l, m, X, Y, Z):
    """SphericalHarmonics::Y (spherical_harmonics.cpp:60-110) at lattice
    points; NaN at the origin, as acos(0/0)."""
    mm = abs(m)
    with np.errstate(invalid="ignore", divide="ignore"):
        r = np.sqrt(X * X + Y * Y + Z * Z)
        th = np.arccos(Z / r)
    ph = np.arctan2(Y, X)
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) *
                     math.factorial(l - mm) / math.factorial(l + mm))
    res = (-1.0) ** mm * norm * _legendre(l, mm, np.cos(th)) * \
        np.exp(1j * mm * ph)
    return (-1.0) ** mm * np.conj(res) if m < 0 else res


def multipole(l, m, rho, n, a):
    """SphericalHarmonics::Q (spherical_harmonics.cpp:116-134):
    int conj(Y_lm) rho r^l with trapezoid weights."""
    X, Y, Z, _ = _coords(n, a)
    r = np.sqrt(X * X + Y * Y + Z * Z)
    f = np.conj(ylm(l, m, X, Y, Z)) * rho * r ** l
    h = 2.0 * a / (n - 1)
    return complex(np.sum(_trap(n) * f) * h ** 3)


def _axis2(rho, n, a, axis):
    X, Y, Z, _ = _coords(n, a)
    c = (X, Y, Z)[axis]
    return float(np.sum(c * c * rho) / np.sum(rho))


# --- the writer --------------------------------------------------------------

def nuclear_data(arr, n, a, A, Z, obs_n=None, obs_p=None):
    """sqrt<x^2>, <y^2>, <z^2>, RN, RP, CR, betaReal as the log prints them
    (output.cpp:160-198; iteration_data.cpp:38-151)."""
    rho_n, rho_p = arr["rho_n"], arr["rho_p"]
    rho = rho_n + rho_p
    X, Y, Z3, _ = _coords(n, a)
    r2 = X * X + Y * Y + Z3 * Z3
    d = {"x2": _axis2(rho, n, a, 0), "y2": _axis2(rho, n, a, 1),
         "z2": _axis2(rho, n, a, 2)}
    d["rn2"] = integral(r2 * rho_n, n, a) / integral(rho_n, n, a)
    d["rp2"] = integral(r2 * rho_p, n, a) / integral(rho_p, n, a)
    radius = integral(r2 * rho, n, a) / integral(rho, n, a)
    a20 = multipole(2, 0, rho, n, a).real
    beta = 4 * math.pi * a20 / (5 * A * radius)
    if d["x2"] > d["z2"]:
        beta = -beta
    d["beta_real"] = beta
    if obs_n is not None and obs_p is not None:
        # chargeRadius(psiN, psiP, N, Z) called with N = Z_in, Z = A - Z_in
        # (output.cpp:107-108, 186-188)
        n_arg, z_arg = Z, A - Z
        corr = sum(MU_N * o[4] / HBAR ** 2 for o in obs_n)
        corr += sum(MU_P * o[4] / HBAR ** 2 for o in obs_p)
        corr *= 2.0 * (HBAR * HBAR / MASS / MASS) / z_arg
        d["cr2"] = abs(d["rp2"] + n_arg * RN2 / z_arg + RP2 + corr)
    return d


def localisation(tau, rho, grad):
    """The localisation function C of output.cpp:326-355."""
    tf = 3.0 / 5.0 * (3 * math.pi ** 2) ** (2.0 / 3.0) * np.power(rho, 5.0 / 3.0)
    g2 = np.sum(np.asarray(grad) ** 2, axis=1)
    return 1.0 / (1.0 + np.power((tau * rho - 0.25 * g2) /
                                 (rho * tf + 1e-12), 2))


def write(folder, name, data, cfg, res, arr, shells=None, log=(),
          cpu_time=None, append=False):
    """Writes the output step's files for one finished run.

    data: the run's JSON input (dict); cfg: the abi.HFConfig it was run
    with; res, arr: hf_run(cfg, outputs=True); shells: (classified neutron
    states, classified proton states, neutron obs, proton obs) or None to
    compute them with ncgm_shell_observables; log: the input's "log" list;
    append: the reference's mode 'a' for the energy CSVs."""
    n, a = cfg.n, cfg.box_size / 2.0
    h = 2.0 * a / (n - 1)
    A, Z = cfg.A, cfg.Z
    if shells is None:
        from . import Context, Grid, shell_observables
        ctx = Context(Grid(n, a), max(arr["orbitals_n"].shape[1],
                                      arr["orbitals_p"].shape[1], 1))
        obs_n = shell_observables(ctx, arr["orbitals_n"])
        obs_p = shell_observables(ctx, arr["orbitals_p"])
        ctx.close()
        shells = (classify(obs_n), classify(obs_p), obs_n, obs_p)
    sh_n, sh_p, obs_n, obs_p = shells
    nd = nuclear_data(arr, n, a, A, Z, obs_n, obs_p)
    rho = arr["rho_n"] + arr["rho_p"]
    t = arr["terms"]
    e_int = float(res.E_int)
    spe2 = float(np.sum(arr["spe_n"]) + np.sum(arr["spe_p"]))
    os.makedirs(folder, exist_ok=True)
    L = []
    L.append("Threads used: 1")
    L.append("=== BOX ===")
    L.append("Size: [-%s, %s] fm " % (fmt(a), fmt(a)))
    L.append("Steps: %d" % n)
    L.append("Step size: %s fm" % fmt(h))
    L.append("")
    L.append("=== NUCLEUS ===")
    L.append("Z = %d, A = %d" % (Z, A))
    L.append("")
    yes = lambda v: "YES" if v else "NO"
    L.append("=== Functional ===")
    L.append("Name: %s" % json.dumps(data.get("functional", "")))
    L.append("Options: J2 terms: %s | Spin orbit: %s | Coulomb: %s" % (
        yes(cfg.use_j), yes(cfg.spin_orbit),
        yes(cfg.use_coulomb)))
    L.append("")
    L.append("=== Nuclear data ===")
    L.append("sqrt<x^2>: %s fm, sqrt<y^2>: %s fm, sqrt<z^2>: %s fm" % (
        fmt(math.sqrt(nd["x2"])), fmt(math.sqrt(nd["y2"])),
        fmt(math.sqrt(nd["z2"]))))
    L.append("RN: %s fm" % fmt(math.sqrt(nd["rn2"])))
    L.append("RP: %s fm" % fmt(math.sqrt(nd["rp2"])))
    L.append("CR: %s fm" % fmt(math.sqrt(nd["cr2"])))
    L.append("")
    L.append("Beta2: %s" % fmt(res.beta))
    L.append("Beta2 computed from physical radius: %s" % fmt(nd["beta_real"]))
    L.append("")
    L.append("=== Convergence ===")
    L.append("Iterations: %d" % res.iterations)
    L.append("Energy tolerance: %s MeV" % fmt(cfg.energy_tol))
    L.append("CPU time: %s s" % fmt(res.wall_s if cpu_time is None
                                    else cpu_time))
    L.append("")
    L.append("=== Density Functional contributions ===")
    for lab, v in zip(abi.ENERGY_TABLE_LABELS[:15], t[:15]):
        L.append("%s: %s MeV" % (lab, fmt(v)))
    L.append("E_INT: %s MeV" % fmt(e_int))
    L.append("")
    L.append("=== HF Energy ===")
    L.append("E (SPE): %s MeV" % fmt(spe2))
    L.append("E (REA): %s MeV" % fmt(t[15]))
    L.append("E_HF: %s MeV" % fmt(res.E_HF))
    L.append("")
    L.append("E_INT/E_HF - 1: %s %%" % fmt(100.0 * (e_int / res.E_HF - 1.0)))
    L.append("")
    L.append("=== Lagrange derivatives recomputed data ===")
    L.append("Lagrange recomputed energy: %s MeV" % fmt(res.E_int_lagrange))
    L.append("")
    L.append("=== Neutrons SP states ===")
    L.append(shells_table(sh_n, arr["spe_n"]))
    L.append("")
    L.append("=== Protons SP states ===")
    L.append(shells_table(sh_p, arr["spe_p"]))
    L.append("")
    L.append("=== Multipole moments ===")
    l_max = -1
    for s in log:
        if s.startswith("multipoles_") and s[11:].isdigit():
            l_max = int(s[11:])
            break
    for l in range(0, min(l_max, 5) + 1) if l_max > 0 else ():
        L.append("l: %d" % l)
        for m in range(-l, l + 1):
            q = multipole(l, m, rho, n, a)
            L.append("%d, %d: (%s,%s)" % (l, m, fmt(q.real), fmt(q.imag)))
        L.append("")
    with open(os.path.join(folder, name + "_log.txt"), "a") as f:
        f.write("\n".join(L) + "\n")

    outdir = os.path.join(folder, name + "_output")
    ddir = os.path.join(outdir, "data")
    fdir = os.path.join(outdir, "fields")
    os.makedirs(ddir, exist_ok=True)
    os.makedirs(fdir, exist_ok=True)
    mode = "a" if append else "w"
    en = np.asarray(arr["energies"])
    for key, col, fname in (("tot_energies", 0, "int_energies.csv"),
                            ("hf_energies", 1, "hf_energies.csv")):
        if key in log:
            with open(os.path.join(ddir, fname), mode) as f:
                for v in en[:, col]:
                    f.write("%.16g\n" % v)
    write_matrix(os.path.join(fdir, "density.csv"), rho)
    write_matrix(os.path.join(fdir, "density_n.csv"), arr["rho_n"])
    write_matrix(os.path.join(fdir, "density_p.csv"), arr["rho_p"])
    write_matrix(os.path.join(fdir, "kinetic_n.csv"), arr["tau_n"])
    write_matrix(os.path.join(fdir, "kinetic_p.csv"), arr["tau_p"])
    write_matrix(os.path.join(fdir, "Field_n.csv"), arr["U_n"])
    write_matrix(os.path.join(fdir, "Field_p.csv"), arr["U_p"])
    write_matrix(os.path.join(fdir, "nabla2rho_n.csv"), arr["grad_rho_n"])
    write_matrix(os.path.join(fdir, "nabla2rho_p.csv"), arr["grad_rho_p"])
    tau = arr["tau_n"] + arr["tau_p"]
    grad = arr["grad_rho_n"] + arr["grad_rho_p"]
    write_matrix(os.path.join(fdir, "C_p.csv"),
                 localisation(arr["tau_p"], arr["rho_p"], arr["grad_rho_p"]))
    write_matrix(os.path.join(fdir, "C.csv"), localisation(tau, rho, grad))
    write_matrix(os.path.join(fdir, "C_n.csv"),
                 localisation(arr["tau_n"], arr["rho_n"], arr["grad_rho_n"]))

    # data.json: one entry appended (keys sorted, 4-space indent)
    entry = {"beta": float(res.beta), "betaReal": float(nd["beta_real"]),
             "EintLag": float(res.E_int_lagrange), "Eint": e_int,
             "EpairN": float(res.E_pair_n), "EpairP": float(res.E_pair_p),
             "gamma": float(res.gamma) * 180.0 / math.pi, "a": float(a),
             "iter": int(res.iterations),
             "constraintsEnergy": float(arr["constraints_energy"]),
             "step": float(h)}
    jpath = os.path.join(ddir, "data.json")
    doc = {}
    if os.path.exists(jpath):
        try:
            with open(jpath) as f:
                doc = json.load(f)
        except (ValueError, OSError):
            doc = {}
    if not isinstance(doc.get("data"), list):
        doc["data"] = []
    doc["data"].append(entry)
    with open(jpath, "w") as f:
        json.dump(doc, f, indent=4, sort_keys=True)
    return nd
