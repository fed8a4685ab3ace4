"""Run configuration: the reference's JSON input schema mapped onto
ncgm_hf_config.

Mirrors InputParser (src/system/input_parser.cpp:50-261) and its validity
check (7-48): the same keys, the same defaults, the same rejections (raised as
ValueError instead of printed and skipped). Skyrme functionals are converted
to EDF coupling constants exactly as EDF::setFromInteraction
(src/skyrme/EDF.cpp:61-103) does.
"""
from __future__ import annotations

from . import abi

# Published Skyrme parameter sets used by the benchmark configurations, in the
# reference's functional-file keys (functionals/<name>.json). Values are the
# standard parameterisations: SLy4 (Chabanat et al., Nucl. Phys. A 635 (1998)
# 231) and SkM* (Bartel et al., Nucl. Phys. A 386 (1982) 79), with the
# reference's optional flags (SLy4 switches the J^2 terms off).
FUNCTIONALS = {
    "SLy4": {"J2": False, "t0": -2488.91, "t1": 486.82, "t2": -546.39,
             "t3": 13777.0, "W0": 123.0, "x0": 0.834, "x1": -0.344,
             "x2": -1.0, "x3": 1.354, "sigma": 0.16666666},
    "SKMstar": {"t0": -2645.0, "t1": 410.0, "t2": -135.0, "t3": 15595.0,
                "W0": 130.0, "x0": 0.09, "x1": 0.0, "x2": 0.0, "x3": 0.0,
                "sigma": 0.16666666},
}

# parameters/woods_saxon.json and parameters/minimization_parameters.json
WOODS_SAXON = {"V0": 55.5, "r0": 1.20, "diffusivity": 0.67,
               "so_V0": 55.5, "kappa": 0.86}
WS_GCG = {"maxIter": 10, "tol": 1e-2, "steps": 40, "cgTol": 1e-4}
HF_GCG = {"maxIter": 1, "tol": 1e-6, "steps": 80, "cgTol": 1e-5}


def edf_from_skyrme(p: dict) -> abi.Edf:
    """EDF::EDF + setFromInteraction (src/skyrme/EDF.cpp:4-103)."""
    if "t0" not in p:
        return abi.Edf(*[p[k] for k in (
            "C0rr", "C1rr", "C0Drr", "C1Drr", "C0rt", "C1rt", "C0J2", "C1J2",
            "C0rdr", "C1rdr", "C0nJ", "C1nJ", "sigma")])
    W0 = p["W0"]
    W0_pr = p.get("W0_pr", W0)
    te = to = 0.0
    if "te" in p:
        te, to = p["te"], p["to"]
    elif "aT" in p:
        to = 4 * p["aT"] / 5
        te = 8 * p["bT"] / 5 - to
    t0, t1, t2, t3 = p["t0"], p["t1"], p["t2"], p["t3"]
    x0, x1, x2, x3 = p["x0"], p["x1"], p["x2"], p["x3"]
    e = abi.Edf()
    e.sigma = p["sigma"]
    e.C0rr = 3 * t0 / 8
    e.C1rr = -t0 * (0.5 + x0) / 4
    e.C0Drr = 3 * t3 / 48
    e.C1Drr = -t3 * (0.5 + x3) / 24
    e.C0rt = 3 * t1 / 16 + t2 * (5.0 / 4.0 + x2) / 4
    e.C1rt = -t1 * (0.5 + x1) / 8 + t2 * (0.5 + x2) / 8
    e.C0rdr = -9 * t1 / 64 + t2 * (5.0 / 4.0 + x2) / 16
    e.C1rdr = 3 * t1 * (0.5 + x1) / 32 + t2 * (0.5 + x2) / 32
    e.C0nJ = -0.5 * W0 - 0.25 * W0_pr
    e.C1nJ = -0.5 * W0
    C0T = -(t1 * (1 - 2 * x1) - t2 * (1 + 2 * x2)) / 16
    C1T = -(t1 - t2) / 16
    C0F = -3 * (te + 3 * to) / 8
    C1F = -3 * (te - to) / 8
    e.C0J2 = -0.5 * (C0T - 0.5 * C0F)
    e.C1J2 = -0.5 * (C1T - 0.5 * C1F)
    return e


def _gcg(d: dict, precision: int = abi.FP64) -> abi.GcgParams:
    return abi.GcgParams(max_iter=d["maxIter"], tol=d["tol"],
                         cg_steps=d["steps"], cg_tol=d["cgTol"], shift=0.0,
                         ordering=abi.ORDER_ASCENDING, precision=precision,
                         precond=0)


def _pairing(block: dict, n_particles: int, window_default=5.0):
    return abi.Pairing(V0=float(block["V0"]),
                       window=float(block.get("window", window_default)),
                       basis_size=int(block["HFbasisSize"]),
                       window_both=int(block.get("windowBoth", True)),
                       active=1)


def from_input(data: dict, functional: dict | None = None,
               precision: int = abi.FP64) -> abi.HFConfig:
    """InputParser (src/system/input_parser.cpp:50-261) for one input dict."""
    cfg = abi.HFConfig()
    A, Z = int(data["nucleus"]["A"]), int(data["nucleus"]["Z"])
    N = A - Z
    cfg.A, cfg.Z = A, Z
    cfg.n = int(data["box"]["axisMeshPoints"])
    cfg.box_size = float(data["box"]["boxSize"])
    fun = functional if functional is not None else FUNCTIONALS[data["functional"]]
    cfg.edf = edf_from_skyrme(fun)

    def opt(field):  # setInteractionOptionalField (input_parser.cpp:227-236)
        if field in fun:
            return bool(fun[field])
        if field in data:
            return bool(data[field])
        return True
    cfg.use_j = int(opt("J2"))
    cfg.spin_orbit = int(opt("spinOrbit"))
    cfg.com_corr = int(opt("COMCorrection"))
    cfg.use_coulomb = int(data.get("coulombInteraction", True))
    cfg.start_hfb_iter = int(data.get("startHFBIter", 3))
    cfg.constrain_com = int(data.get("constrainCOM", False))
    # "constraints": [{"l", "m", "target"}] (input_parser.cpp:189-196)
    mps = data.get("constraints", [])
    if len(mps) > abi.MAX_MULTIPOLE:
        raise ValueError("at most %d multipole constraints" % abi.MAX_MULTIPOLE)
    cfg.n_multipole = len(mps)
    for i, c in enumerate(mps):
        l, m = int(c["l"]), int(c["m"])
        if l < 0 or l > 9 or abs(m) > l:
            raise ValueError("multipole constraint needs 0 <= l <= 9, |m| <= l")
        cfg.mp_l[i], cfg.mp_m[i] = l, m
        cfg.mp_target[i] = float(c["target"])
    cfg.constraints_tol = float(data.get("constraintsTol", 1e-3))
    cfg.pairing_threshold = float(data.get("pairingThreshold", 1e-3))
    cfg.density_mix = float(data.get("densityMix", 0.25))
    cfg.max_iterations = int(data["maxIterations"])
    cfg.energy_tol = float(data["energyTol"])
    cfg.ws_V0 = WOODS_SAXON["V0"]
    cfg.ws_r0 = WOODS_SAXON["r0"]
    cfg.ws_diff = WOODS_SAXON["diffusivity"]
    cfg.ws_kappa = WOODS_SAXON["kappa"]
    cfg.wsso_V0 = WOODS_SAXON["so_V0"]
    cfg.ws_gcg = _gcg(WS_GCG)
    cfg.hf_gcg = _gcg(HF_GCG, precision)
    cfg.pairing_type = abi.PAIRING_NONE
    cfg.pair_n = abi.Pairing()
    cfg.pair_p = abi.Pairing()
    pd = data.get("pairing")
    if pd is not None:
        t = pd["type"]
        cfg.pairing_type = {"HFB": abi.PAIRING_HFB,
                            "BCS": abi.PAIRING_BCS}.get(t, abi.PAIRING_NONE)
        if "neutron" in pd:
            cfg.pair_n = _pairing(pd["neutron"], N)
        if "proton" in pd:
            cfg.pair_p = _pairing(pd["proton"], Z)
        if "neutron" not in pd and "proton" not in pd:
            bn = pd.get("HFbasisSizeN", pd.get("HFbasisSize"))
            bp = pd.get("HFbasisSizeP", pd.get("HFbasisSize"))
            for attr, b in (("pair_n", bn), ("pair_p", bp)):
                setattr(cfg, attr, abi.Pairing(
                    V0=float(pd["V0"]), window=float(pd["window"]),
                    basis_size=int(b),
                    window_both=int(pd.get("windowBoth", True)), active=1))
    if "deformation" in data:
        d = data["deformation"]
        cfg.initial_beta = float(d.get("guess", d["start"]))
    else:
        cfg.initial_beta = float(data.get("initialBeta2", 0.0))
    cfg.beta3 = float(data.get("beta3", 0.0))
    check(cfg)
    return cfg


def check(cfg: abi.HFConfig) -> None:
    """InputParser::check (src/system/input_parser.cpp:7-48)."""
    if cfg.A % 2 or cfg.Z % 2:
        raise ValueError("Nucleus must be even-even")
    if cfg.A < cfg.Z:
        raise ValueError("Nucleus A must be larger than Z")
    if cfg.pairing_type != abi.PAIRING_NONE:
        N = cfg.A - cfg.Z
        if cfg.pair_n.V0 < 0 or cfg.pair_p.V0 < 0:
            raise ValueError("Pairing strength must be positive")
        addN = cfg.pair_n.basis_size - N
        addP = cfg.pair_p.basis_size - cfg.Z
        if addN <= 0:
            raise ValueError("Neutron HF basis size must be larger than "
                             "particle number")
        if addP <= 0:
            raise ValueError("Proton HF basis size must be larger than "
                             "particle number")
        if addN % 2 or addP % 2:
            raise ValueError("HF basis size must be even")
    if cfg.n % 2:
        raise ValueError("Mesh points must be even")


def curve_points(A: int, start: float, end: float, count: int):
    """Quadrupole targets mu20 = beta * 3 A R^2 / (4 pi), R = 1.2 A^(1/3)
    (Utilities::mu20FromBeta, src/util/utilities.cpp:71-73)."""
    import math
    R0 = 1.2 * A ** (1.0 / 3.0)
    if count == 1:
        betas = [start]
    else:
        betas = [start + (end - start) * i / (count - 1) for i in range(count)]
    return [(b, b * 3 * A * R0 * R0 / 4 / math.pi) for b in betas]


def orbital_counts(cfg: abi.HFConfig):
    """Columns per species (main.cpp:67-68)."""
    N = cfg.A - cfg.Z
    if cfg.pairing_type == abi.PAIRING_NONE:
        return N, cfg.Z
    on = cfg.pair_n.basis_size if cfg.pair_n.active else N
    op = cfg.pair_p.basis_size if cfg.pair_p.active else cfg.Z
    return on, op
