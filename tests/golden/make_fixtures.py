"""Golden fixtures for the GPU parity tests at the benchmark lattices.

Runs the FP64 CPU oracle (a restatement of the reference's run loop,
src/main.cpp:199-342 with IterationData::updateQuantities,
src/util/iteration_data.cpp:852-1125) to its fixed point and stores what
the parity tests compare: E_int, E_HF, every single-particle energy and the
neutron and proton densities. The GPU tests (tests/test_gpu_fixtures.py)
rebuild the same configuration from the stored input and compare.

Each case runs a fixed number of HF iterations (energyTol 0) with a tight
PCG tolerance, so that the stored point is the fixed point itself to far
below the compared tolerances (E 1 keV, levels 1e-5 MeV, densities
1e-7 fm^-3), not wherever the reference's |dE| < 1 keV rule happens to stop.
The densities are stored as float32: the rounding (below 1e-8 fm^-3 for
densities up to 0.17 fm^-3) is an order of magnitude inside the 1e-7 fm^-3
tolerance.

  python tests/golden/make_fixtures.py [case ...]     (default: every case)

The oracle uses every host core (OpenMP). Approximate cost on 8 cores:
o16 a few minutes per hundred iterations, ca40 and the mg24 points longer.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

O16 = {"functional": "SLy4", "nucleus": {"A": 16, "Z": 8},
       "box": {"boxSize": 18.0, "axisMeshPoints": 30}}
CA40 = {"functional": "SLy4", "nucleus": {"A": 40, "Z": 20},
        "box": {"boxSize": 20.0, "axisMeshPoints": 36}}
MG24 = {"functional": "SKMstar", "nucleus": {"A": 24, "Z": 12},
        "box": {"boxSize": 20.0, "axisMeshPoints": 32},
        "pairing": {"type": "BCS", "HFbasisSize": 24, "V0": 300.0,
                    "window": 5.0}}

# The 16-point beta2 grid of the 24Mg deformation curve: (start, end, count)
MG24_CURVE = (-0.3, 0.5, 16)

# name -> (input, HF iterations, PCG tolerance, index on the 24Mg curve or
# None)
CASES = {
    # 16O, SLy4, 30^3, box 18 fm (h = 0.621 fm), 8 + 8 orbitals, Coulomb
    "o16_sly4_n30": (O16, 500, 1e-8, None),
    # 40Ca, SLy4, 36^3, box 20 fm (h = 0.571 fm), 20 + 20 orbitals
    "ca40_sly4_n36": (CA40, 400, 1e-8, None),
    # 24Mg, SkM*, 32^3, box 20 fm, HF+BCS with 24 states per isospin, at
    # points 0, 4 and 15 of the curve (beta2 = -0.3, -0.0867, 0.5) with the
    # curve-mode constraint set. The paired points near the spherical shape
    # converge slowly (point 4 still moves by 2e-5 MeV per iteration after
    # 400 iterations, point 7 likewise), so point 4 runs 1200.
    "mg24_skm_n32_p00": (MG24, 400, 1e-8, 0),
    "mg24_skm_n32_p04": (MG24, 1200, 1e-8, 4),
    "mg24_skm_n32_p15": (MG24, 400, 1e-8, 15),
}


def curve_configs(inp, precision=None, energy_tol=1e-3, max_iterations=500):
    """The 16 constrained configurations of the 24Mg curve, each a cold
    start at its own beta2 (main.cpp:176-185 with mu20 from
    Utilities::mu20FromBeta, utilities.cpp:71-73)."""
    from nuclearcgm_gb300 import abi, config
    A = inp["nucleus"]["A"]
    data = dict(inp, maxIterations=max_iterations, energyTol=energy_tol)
    cfgs = []
    for beta, mu in config.curve_points(A, *MG24_CURVE):
        c = config.from_input(data, precision=abi.FP64 if precision is None
                              else precision)
        c.curve_mode = 1
        c.mu20 = mu
        c.initial_beta = beta
        cfgs.append(c)
    return cfgs


def make_config(inp, iterations, cg_tol, point, precision=None):
    """The abi.HFConfig of a case (shared with the GPU tests)."""
    from nuclearcgm_gb300 import abi, config
    if point is not None:
        cfg = curve_configs(inp, precision, 0.0, iterations)[point]
    else:
        data = dict(inp, maxIterations=iterations, energyTol=0.0)
        cfg = config.from_input(data, precision=abi.FP64 if precision is None
                                else precision)
    cfg.hf_gcg.cg_tol = cg_tol
    return cfg


def path(name):
    return os.path.join(HERE, name + ".npz")


def load(name):
    """The stored fixed point of a case as a dict."""
    z = np.load(path(name))
    d = {k: z[k] for k in z.files}
    d["input"] = json.loads(str(d["input"]))
    return d


def run(name):
    from oracle import oracle
    inp, iters, cg_tol, point = CASES[name]
    cfg = make_config(inp, iters, cg_tol, point)
    t = time.time()
    res, out = oracle.hf_run(cfg)
    secs = time.time() - t
    en = out["energies"]
    np.savez(path(name),
             input=json.dumps(inp), iterations=res.iterations,
             cg_tol=cg_tol, curve_point=-1 if point is None else point,
             E_int=res.E_int, E_HF=res.E_HF, last_dE=res.last_dE,
             beta=res.beta, E_pair_n=res.E_pair_n, E_pair_p=res.E_pair_p,
             spe_n=out["spe_n"], spe_p=out["spe_p"],
             rho_n=out["rho_n"].astype(np.float32),
             rho_p=out["rho_p"].astype(np.float32),
             energies=en, oracle_seconds=secs,
             threads=os.environ.get("OMP_NUM_THREADS", str(os.cpu_count())))
    tail = np.abs(np.diff(en[-20:, 0])).max() if len(en) > 20 else np.nan
    print("%s: %d iterations in %.0f s, E_int %.9f E_HF %.9f, last dE %.2e,"
          " max |dE| over the last 20 iterations %.2e" % (
              name, res.iterations, secs, res.E_int, res.E_HF, res.last_dE,
              tail), flush=True)


if __name__ == "__main__":
    for name in sys.argv[1:] or list(CASES):
        run(name)
