"""CPU checks of the C-ABI boundary: the library builds, loads and exports
every entry point declared in include/ncgm.h; no compute calls."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "ncgm.h")).read()
    return sorted(set(re.findall(r"\b(ncgm_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_exports_every_declared_symbol():
    from nuclearcgm_gb300 import build, abi
    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(ncgm_[a-z0-9_]+)", out))
    declared = _declared()
    assert declared, "no declarations parsed"
    missing = [s for s in declared if s not in exported]
    assert not missing, "not exported: %s" % missing
    # the Python binding table covers the same set
    assert set(abi.SIGNATURES) == set(declared)


def test_library_loads_and_binds():
    import nuclearcgm_gb300 as ng
    lib = ng.load()
    for name in ng.abi.SIGNATURES:
        assert hasattr(lib, name)
    assert isinstance(lib.ncgm_last_error(), bytes)


def test_no_device_is_reported_as_status_not_crash():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is visible")
    import nuclearcgm_gb300 as ng
    with pytest.raises(ng.NcgmError) as e:
        ng.Context(ng.Grid(8, 3.5), 4)
    assert e.value.status == 2  # NCGM_ERR_CUDA


def test_edf_conversion_matches_python_restatement():
    import ctypes as C
    import nuclearcgm_gb300 as ng
    from nuclearcgm_gb300 import abi, config
    p = config.FUNCTIONALS["SLy4"]
    sk = abi.Skyrme(W0=p["W0"], W0_pr=p["W0"], t0=p["t0"], t1=p["t1"],
                    t2=p["t2"], t3=p["t3"], x0=p["x0"], x1=p["x1"],
                    x2=p["x2"], x3=p["x3"], sigma=p["sigma"], te=0, to=0)
    out = abi.Edf()
    assert ng.load().ncgm_edf_from_skyrme(C.byref(sk), C.byref(out)) == 0
    ref = config.edf_from_skyrme(p)
    for name, _ in abi.Edf._fields_:
        assert getattr(out, name) == pytest.approx(getattr(ref, name),
                                                   rel=1e-15)
    # SLy4 textbook couplings
    assert ref.C0rr == pytest.approx(3 * -2488.91 / 8)
    assert ref.C1nJ == pytest.approx(-61.5)
