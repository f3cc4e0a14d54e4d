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
