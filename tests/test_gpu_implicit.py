"""ImplicitTYMSolver (SU(2), SU(3)) on the GPU against the oracle, through the C ABI:
fields within 1e-10 after the run for the pure gauge field with an active
region, and within 1e-9 with super particles at dt = a, one particle per cell
(temporal optimized implicit cgc ngp, with the reference's current shift for
that case)."""
import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N
from tests.helpers import oracle_ic, fresh, link_rel_err, field_rel_err

pytestmark = pytest.mark.gpu


def to_handle(g):
    h = opx.Handle(2, g.dims, a=g.a, dt=g.dt, g=g.g)
    for f, arr in ((N.FIELD_U, g.U), (N.FIELD_UNEXT, g.Unext), (N.FIELD_E, g.E)):
        h.upload(f, arr)
    return h


@pytest.mark.parametrize("iters,damp", [(0, 0.0), (3, 0.0), (4, 0.25)])
def test_implicit_pure_gauge(native, orc, iters, damp):
    g = fresh(oracle_ic(2, (8, 6, 10), 21, 0.3, 0.2, dt=0.1))
    act = np.ones(g.V, np.uint8)
    act[: 60] = 0
    g.active[:] = act
    h = to_handle(g)
    h.set_active(act)
    h.set_field_solver(N.SOLVER_IMPLICIT, iters, damp)
    sim = orc.OracleSimulation(g, implicit=(iters, damp))
    sim.initialize()
    h.initialize()
    for _ in range(6):
        sim.step()
        h.step(1)
    assert link_rel_err(h.download(N.FIELD_U), g.U) <= 1e-10
    assert link_rel_err(h.download(N.FIELD_UNEXT), g.Unext) <= 1e-10
    assert field_rel_err(h.download(N.FIELD_E), g.E) <= 1e-10


def test_implicit_with_super_particles_dt_equals_a(native, orc):
    """dt = a amplifies rounding quickly: in the oracle itself a 1e-15 relative
    change of E grows to 2.2e-11 per link in these 5 steps, so the device's own
    rounding (exp, pow) is held to 1e-9 here."""
    from oracle import cgc
    nuclei = [cgc.MVNucleus(orientation=1, location=12.0, width=1.5, mu=0.5, seed=3),
              cgc.MVNucleus(orientation=-1, location=28.0, width=1.5, mu=0.5, seed=4)]
    g = orc.OracleGrid(2, (40, 6, 6), dt=1.0)
    groups, _ = cgc.cgc_mv_super(g, nuclei)
    h = to_handle(g)
    h.set_field_solver(N.SOLVER_IMPLICIT, 3, 0.1)
    for G in groups:
        h.super_upload(G.orientation, G.n, G.base, G.Q[:, :G.n])
    sim = cgc.OracleSuperSimulation(g, groups, implicit=(3, 0.1))
    sim.initialize()
    h.initialize()
    for _ in range(5):
        sim.step()
        h.step(1)
    assert link_rel_err(h.download(N.FIELD_U), g.U) <= 1e-9
    assert field_rel_err(h.download(N.FIELD_E), g.E) <= 1e-9
    J = g.J
    assert np.abs(h.download(N.FIELD_J) - J).max() <= 1e-9 * max(np.abs(J).max(), 1e-30)


@pytest.mark.parametrize("iters,damp", [(0, 0.0), (3, 0.2)])
def test_implicit_su3_vs_oracle(native, orc, iters, damp):
    """SU(3) (SU3GroupElement.pow through the matrix logarithm): fields within
    1e-10 of the oracle after 4 steps, with an active region."""
    g = fresh(oracle_ic(3, (6, 5, 7), 23, 0.25, 0.2, dt=0.1))
    act = np.ones(g.V, np.uint8)
    act[: 30] = 0
    g.active[:] = act
    h = opx.Handle(3, g.dims, a=g.a, dt=g.dt, g=g.g)
    for f, arr in ((N.FIELD_U, g.U), (N.FIELD_UNEXT, g.Unext), (N.FIELD_E, g.E)):
        h.upload(f, arr)
    h.set_active(act)
    h.set_field_solver(N.SOLVER_IMPLICIT, iters, damp)
    sim = orc.OracleSimulation(g, implicit=(iters, damp))
    sim.initialize()
    h.initialize()
    for _ in range(4):
        sim.step()
        h.step(1)
    assert link_rel_err(h.download(N.FIELD_U), g.U) <= 1e-10
    assert link_rel_err(h.download(N.FIELD_UNEXT), g.Unext) <= 1e-10
    assert field_rel_err(h.download(N.FIELD_E), g.E) <= 1e-10