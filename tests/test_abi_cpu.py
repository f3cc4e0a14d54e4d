"""CPU checks of the C ABI: the library builds for sm_103a, loads, exports every
symbol include/opixi.h declares, and fails with a status code (no crash) when no
GPU is usable.  No kernel runs here."""
import os
import re

import pytest

from openpixi_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "opixi.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(opx_[a-z_]+)\s*\(", txt)))


def test_header_matches_binding_list():
    assert header_symbols() == sorted(N.EXPORTED)


def test_library_exports_every_symbol(native):
    for name in header_symbols():
        assert hasattr(native, name), name


def test_library_is_sm103a(native):
    # the fat binary must hold sm_103a code: check the build flags in the recipe
    from openpixi_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)


def test_create_without_gpu_reports_error(native):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(N.OpixiError) as e:
        N.Handle(2, (4, 4, 4))
    assert e.value.code in (N.OPX_ERR_CUDA, N.OPX_ERR_INVALID)


def test_invalid_config_rejected_before_device(native):
    for kw in ({"ncolors": 4, "dims": (4, 4, 4)}, {"ncolors": 2, "dims": (0, 4, 4)},
               {"ncolors": 2, "dims": (4, 4, 4), "dt": -1.0}):
        with pytest.raises(N.OpixiError) as e:
            N.Handle(**kw)
        assert e.value.code == N.OPX_ERR_INVALID


def test_java_double_format():
    """Double.toString as documented in the Java SE API (plain decimal between
    1e-3 and 1e7, otherwise computerized scientific notation)."""
    from openpixi_gb300.diagnostics import java_double as j
    assert j(100.0) == "100.0" and j(0.001) == "0.001" and j(1.0e-4) == "1.0E-4"
    assert j(1.0e7) == "1.0E7" and j(9999999.0) == "9999999.0" and j(-3.5e-4) == "-3.5E-4"
    assert j(0.0) == "0.0" and j(1.0 / 3.0) == "0.3333333333333333" and j(123456789.0) == "1.23456789E8"


def test_measured_loop_selection_and_rows(tmp_path):
    """Simulation.run hands the updates to opx_step_measured only when
    BulkQuantitiesInTime at every step is the only diagnostic, and
    BulkQuantitiesInTime.record writes the row that calculate would (host
    logic, no device: stand-ins for the simulation and the observables)."""
    import types
    from openpixi_gb300.diagnostics import BulkQuantitiesInTime, EnergyDensity
    from openpixi_gb300.simulation import Simulation
    sim = types.SimpleNamespace(tstep=0.05)
    pick = lambda diags: Simulation._measured_loop(types.SimpleNamespace(tstep=0.05, diagnostics=diags))
    assert pick([BulkQuantitiesInTime(str(tmp_path / "a"), 0.05)])
    assert pick([BulkQuantitiesInTime(str(tmp_path / "a"), 0.05), BulkQuantitiesInTime(str(tmp_path / "b"), 0.04)])
    assert not pick([BulkQuantitiesInTime(str(tmp_path / "a"), 0.1)])  # every second step
    assert not pick([BulkQuantitiesInTime(str(tmp_path / "a"), 0.05), EnergyDensity(str(tmp_path / "e"), 0, 0.05)])
    assert not pick([])
    d = BulkQuantitiesInTime(str(tmp_path / "bulk.txt"), 0.05)
    sim.getTimeStep = lambda: 0.05
    d.initialize(sim)
    o = types.SimpleNamespace(e2_total=1.5, b2_total=0.25, px=0.1, py=-0.2, pz=0.3, gauss=1e-14, rho2=0.0)
    d.record(o, 4)
    lines = (tmp_path / "bulk.txt").read_text().splitlines()
    assert lines[0] == BulkQuantitiesInTime.HEADER
    from openpixi_gb300.diagnostics import java_sci
    assert lines[1].split("\t") == [java_sci(v) for v in (4 * 0.05, 1.5, 0.25, 0.1, -0.2, 0.3, 1e-14, 0.0)]
    assert lines[1].split("\t")[1] == "1.5E0"
