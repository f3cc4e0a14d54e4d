"""The precision form's energy bar at the configured length, and the
EnergyDensity file written from the device.

SU(3) pure Yang-Mills on 32^3 (the crop on which the 128^3 precision workload
is checked against the oracle): FP32 links and E with reunitarisation every 10
steps, 500 steps of dt = 0.05, against the oracle's FP64 FastTYMSolver on the
same projected initial state.  Bar: total energy (E^2 + B^2 of
FieldMeasurements) within 1e-6 relative; Gauss law of the FP32 run below 1e-10.

EnergyDensity (EnergyDensity.java:119-166, file format :15-31): the file the
host writer produces from opx_energy_density reads back as D = 3, N = dims and
the device's values bit for bit, and those agree with the oracle to 1e-12.
"""
import os
import struct
import types

import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N
from openpixi_gb300.diagnostics import EnergyDensity
from helpers import fresh, oracle_ic
from test_gpu_parity import handle_from_oracle

pytestmark = pytest.mark.gpu


def test_su3_fp32_500_steps_energy_against_oracle(native, orc):
    dims = (32, 32, 32)
    h64 = opx.Handle(3, dims, dt=0.05, precision=N.OPX_F64)
    h64.init_random(20261206, 0.2, 0.2)
    it, g2 = h64.gauss_project(1e-26)
    assert g2 < 1e-26
    U0, E0 = h64.download(N.FIELD_U), h64.download(N.FIELD_E)
    h32 = opx.Handle(3, dims, dt=0.05, precision=N.OPX_F32, reunit_every=10)
    h32.upload(N.FIELD_U, U0)
    h32.upload(N.FIELD_E, E0)
    h32.initialize()
    g = orc.OracleGrid(3, dims, dt=0.05)
    g.U[...] = U0
    g.E[...] = E0
    g.update_links()
    nth = max(1, min(64, len(os.sched_getaffinity(0))))
    for _ in range(500):
        g.store_fields()
        g.update_grid_omp(nth)
    h32.step(500)
    b = g.bulk()
    e_ref = b[11] + b[12]
    o = h32.reduce()
    rel = abs(o.e2_total + o.b2_total - e_ref) / e_ref
    assert rel <= 1e-6, rel
    assert o.gauss < 1e-10


def test_energy_density_file_from_device(native, orc, tmp_path):
    g = fresh(oracle_ic(2, (6, 8, 5), 13, 0.3, 0.3, a=(1.0, 1.1, 0.9)))
    h = handle_from_oracle(g)
    sim = orc.OracleSimulation(g)
    sim.initialize()
    h.initialize()
    for _ in range(3):
        sim.step()
        h.step(1)
    grid = types.SimpleNamespace(dims=h.dims, energy_density=h.energy_density)
    w = EnergyDensity(str(tmp_path / "energy.bin"), 0.05, 0.05)
    w.initialize(types.SimpleNamespace(getTimeStep=lambda: 0.05))
    w.calculate(grid, [], 3)
    raw = (tmp_path / "energy_1.bin").read_bytes()
    assert struct.unpack(">4i", raw[:16]) == (3, 6, 8, 5)
    body = np.frombuffer(raw[16:], dtype=">f8").astype(np.float64)
    assert body.size == 6 * 8 * 5
    assert np.array_equal(body, h.energy_density())
    ref = g.energy_density()
    assert np.abs(body - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("nc", [2, 3])
def test_leapfrog_matches_temporal_ym_solver(native, orc, nc):
    """The device leapfrog (FastTYMSolver's staple form) against the oracle's
    TemporalYangMillsSolver (the plaquette form, TemporalYangMillsSolver.java:49-95)
    on an uneven lattice: links and E within 1e-12 per link after 20 steps."""
    from helpers import link_rel_err, field_rel_err
    g = fresh(oracle_ic(nc, (6, 5, 8), 21, 0.3, 0.3, a=(1.0, 0.9, 1.1)))
    h = handle_from_oracle(g)
    t = g.copy()
    t.update_links()
    h.initialize()
    for _ in range(20):
        t.store_fields()
        t.update_grid_tym()
    h.step(20)
    assert link_rel_err(h.download(N.FIELD_U), t.U) <= 1e-12
    assert link_rel_err(h.download(N.FIELD_UNEXT), t.Unext) <= 1e-12
    assert field_rel_err(h.download(N.FIELD_E), t.E) <= 1e-12
