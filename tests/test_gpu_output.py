"""GPU side of the output step: the shell observables against the oracle,
and the writer on a finished run (single-particle classification of 16O)."""
import json

import numpy as np
import pytest

import nuclearcgm_gb300 as ng
from conftest import random_block
from nuclearcgm_gb300 import config, output
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [9, 14])
def test_shell_observables_match_oracle(n):
    a = 0.5 * (n - 1) * 0.9
    ctx = ng.Context(ng.Grid(n, a), 6)
    Phi = np.asfortranarray(random_block(2 * n ** 3, 5, 3 * n))
    got = ng.shell_observables(ctx, Phi)
    ref = oracle.shell_observables(n, a, Phi)
    scale = np.abs(ref).max(axis=0)
    assert np.all(np.abs(got - ref) <= 1e-10 * scale)
    ctx.close()


def test_writer_on_a_converged_run(tmp_path):
    """16O on a 20^3 lattice: the neutron table holds 1s1/2 (2 states),
    1p3/2 (4) and 1p1/2 (2), and data.json carries the run's energies."""
    data = {"functional": "SLy4", "nucleus": {"A": 16, "Z": 8},
            "box": {"boxSize": 16.0, "axisMeshPoints": 20},
            "maxIterations": 200, "energyTol": 1e-6}
    cfg = config.from_input(data)
    res, arr = ng.hf_run(cfg, outputs=True)
    nd = output.write(str(tmp_path), "o16", data, cfg, res, arr,
                      log=["tot_energies"])
    ctx = ng.Context(ng.Grid(cfg.n, cfg.box_size / 2), 8)
    sh = output.classify(ng.shell_observables(ctx, arr["orbitals_n"]))
    ctx.close()
    ls = sorted(s[0] for s in sh)
    js = sorted(s[1] for s in sh)
    par = sorted(1 if s[3] > 0 else -1 for s in sh)
    print("neutron shells (l, j, mj, parity):", sh)
    assert ls == [0.0] * 2 + [1.0] * 6
    assert js == [0.5] * 4 + [1.5] * 4
    assert par == [-1] * 6 + [1] * 2
    doc = json.loads((tmp_path / "o16_output" / "data" / "data.json")
                     .read_text())
    e = doc["data"][-1]
    assert e["Eint"] == res.E_int and e["EintLag"] == res.E_int_lagrange
    assert e["iter"] == res.iterations
    assert 2.0 < np.sqrt(nd["rn2"]) < 3.5 and 2.0 < np.sqrt(nd["cr2"]) < 3.5
    txt = (tmp_path / "o16_log.txt").read_text()
    assert "=== Neutrons SP states ===" in txt and "3/2" in txt
