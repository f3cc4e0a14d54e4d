"""The CUDA path against the committed golden fixtures (tests/golden/*.npz,
written by the oracle through tests/golden/make_golden.py), through the C ABI.
Bars: FP64 fields 1e-10 per link; BulkQuantities and per-slice rows 1e-12 of
their scale (1e-10 for the Poynting rows and the CGC runs, whose initial
conditions carry FFT rounding); particle positions bit-exact; particle charges
1e-10 of the largest."""
import os

import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N
from tests.helpers import link_rel_err, field_rel_err

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


def close(a, b, tol):
    return np.abs(np.asarray(a) - np.asarray(b)).max() <= tol * max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", ["su2_fp64_6cube", "su3_fp64_4x4x6"])
def test_leapfrog_golden(native, name):
    f = load(name)
    h = opx.Handle(int(f["nc"]), tuple(int(x) for x in f["dims"]), a=tuple(f["a"]), dt=float(f["dt"]),
                   g=float(f["g"]))
    h.upload(N.FIELD_U, f["U0"])
    h.upload(N.FIELD_E, f["E0"])
    h.initialize()
    for k in range(int(f["steps"])):
        h.step(1)
        o = h.reduce()
        got = np.array(list(o.e2) + list(o.b2) + [o.px, o.py, o.pz, o.gauss, o.rho2, o.e2_total, o.b2_total])
        ref = f["bulk"][k]
        assert np.all(np.abs(got[:6] - ref[:6]) <= 1e-12 * np.abs(ref[:6]) + 1e-300), k
        # the Gauss column sits at rounding level (mean G^2 ~ 1e-30): absolute bar
        assert abs(got[9] - ref[9]) <= 1e-12 * abs(ref[9]) + 1e-26, k
    assert link_rel_err(h.download(N.FIELD_U), f["U"]) <= 1e-10
    assert link_rel_err(h.download(N.FIELD_UNEXT), f["Unext"]) <= 1e-10
    assert field_rel_err(h.download(N.FIELD_E), f["E"]) <= 1e-10
    assert close(h.energy_density(), f["energy_density"], 1e-12)
    assert close(h.projected_energy(0), f["projected0"], 1e-12)


def test_cpic_golden(native):
    f = load("cpic_su2_12x6x6")
    h = opx.Handle(2, tuple(int(x) for x in f["dims"]), dt=float(f["dt"]))
    h.upload(N.FIELD_U, f["U0"])
    h.upload(N.FIELD_E, f["E0"])
    h.particles_upload(f["p_pos0"], f["p_pos1"], f["p_vel"], f["p_Q0"], f["p_Q1"], f["p_dir"])
    h.initialize()
    h.step(int(f["steps"]))
    assert link_rel_err(h.download(N.FIELD_U), f["U"]) <= 1e-10
    assert field_rel_err(h.download(N.FIELD_E), f["E"]) <= 1e-10
    d = h.particles_download()
    assert same_bits(d["pos0"], f["P_pos0"]) and same_bits(d["pos1"], f["P_pos1"])
    assert close(d["Q0"], f["P_Q0"], 1e-10) and close(d["Q1"], f["P_Q1"], 1e-10)
    assert close(h.download(N.FIELD_RHO), f["rho"], 1e-10)
    assert close(h.download(N.FIELD_J), f["J"], 1e-10)


def test_cgc_golden(native):
    f = load("cgc_su2_20x6x6")
    dims = tuple(int(x) for x in f["dims"])
    h = opx.Handle(2, dims, dt=float(f["dt"]))
    base = {"direction": 0, "width": 1.5, "mu": 0.5, "use_seed": 1, "uvt": 4.44, "coherence": 0.0, "ir": 0.0}
    h.cgc_mv([dict(base, orientation=1, location=6.0, seed=1), dict(base, orientation=-1, location=14.0, seed=2)])
    assert link_rel_err(h.download(N.FIELD_U), f["ic_U"]) <= 1e-10
    assert link_rel_err(h.download(N.FIELD_UNEXT), f["ic_Unext"]) <= 1e-10
    assert field_rel_err(h.download(N.FIELD_E), f["ic_E"]) <= 1e-10
    d = h.particles_download()
    assert same_bits(d["pos0"], f["ic_pos0"]) and same_bits(d["pos1"], f["ic_pos1"])
    assert close(d["Q0"], f["ic_Q0"], 1e-10)
    h.initialize()
    h.step(int(f["steps"]))
    assert link_rel_err(h.download(N.FIELD_U), f["U"]) <= 1e-10
    assert field_rel_err(h.download(N.FIELD_E), f["E"]) <= 1e-10
    d = h.particles_download()
    assert same_bits(d["pos0"], f["P_pos0"])
    assert close(d["Q0"], f["P_Q0"], 1e-10)
    assert close(h.projected_energy(0), f["projected"], 1e-10)
    assert close(h.projected_poynting(0), f["poynting"], 1e-9)
