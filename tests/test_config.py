"""CPU checks of the input-schema mirror (InputParser)."""
import pytest

from nuclearcgm_gb300 import abi, config


def _base(**kw):
    d = {"functional": "SLy4", "nucleus": {"A": 16, "Z": 8},
         "box": {"boxSize": 18.0, "axisMeshPoints": 30},
         "maxIterations": 500, "energyTol": 1e-3}
    d.update(kw)
    return d


def test_defaults_follow_input_parser():
    cfg = config.from_input(_base())
    assert cfg.n == 30 and cfg.box_size == 18.0
    assert cfg.use_coulomb == 1 and cfg.density_mix == 0.25
    assert cfg.start_hfb_iter == 3 and cfg.constraints_tol == 1e-3
    assert cfg.use_j == 0          # SLy4 file sets J2 false
    assert cfg.spin_orbit == 1 and cfg.com_corr == 1
    assert cfg.hf_gcg.max_iter == 1 and cfg.hf_gcg.cg_steps == 80
    assert cfg.ws_gcg.max_iter == 10 and cfg.ws_gcg.cg_tol == 1e-4
    assert config.orbital_counts(cfg) == (8, 8)


def test_pairing_blocks_and_checks():
    d = _base(nucleus={"A": 24, "Z": 12},
              pairing={"type": "BCS", "HFbasisSize": 24, "V0": 300.0,
                       "window": 5.0})
    cfg = config.from_input(d)
    assert cfg.pairing_type == abi.PAIRING_BCS
    assert config.orbital_counts(cfg) == (24, 24)
    bad = _base(nucleus={"A": 24, "Z": 12},
                pairing={"type": "BCS", "HFbasisSize": 12, "V0": 300.0,
                         "window": 5.0})
    with pytest.raises(ValueError):
        config.from_input(bad)
    with pytest.raises(ValueError):
        config.from_input(_base(nucleus={"A": 17, "Z": 8}))
    with pytest.raises(ValueError):
        config.from_input(_base(box={"boxSize": 18.0, "axisMeshPoints": 31}))


def test_curve_points_match_mu20_from_beta():
    pts = config.curve_points(24, -0.3, 0.5, 16)
    assert len(pts) == 16
    import math
    R = 1.2 * 24 ** (1 / 3)
    assert pts[0][1] == pytest.approx(-0.3 * 3 * 24 * R * R / 4 / math.pi)


def test_multipole_constraints_parsed():
    from nuclearcgm_gb300 import abi, config
    data = {"functional": "SLy4", "nucleus": {"A": 16, "Z": 8},
            "box": {"boxSize": 16.0, "axisMeshPoints": 12},
            "maxIterations": 10, "energyTol": 1e-3,
            "constraints": [{"l": 2, "m": 0, "target": 20.0},
                            {"l": 3, "m": -2, "target": 1.5}]}
    cfg = config.from_input(data)
    assert cfg.n_multipole == 2
    assert (cfg.mp_l[0], cfg.mp_m[0], cfg.mp_target[0]) == (2, 0, 20.0)
    assert (cfg.mp_l[1], cfg.mp_m[1], cfg.mp_target[1]) == (3, -2, 1.5)
    import pytest
    with pytest.raises(ValueError):
        config.from_input(dict(data, constraints=[{"l": 1, "m": 2,
                                                   "target": 0.0}]))
    assert abi.MAX_MULTIPOLE == 8
