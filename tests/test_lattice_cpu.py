"""Host-side checks of the lattice geometry helpers (lattice.cuh) that the
kernels share: the site-coordinate division by a multiply and a shift
(div_magic / div_n) against integer division.  Compiled for the host with
nvcc (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_site_coordinate_division(tmp_path):
    nvcc = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
    if not (os.path.exists(nvcc) or shutil.which("nvcc")):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "lattice_div_check")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", os.path.join(HERE, "lattice_div_check.cu"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
