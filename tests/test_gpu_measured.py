"""opx_step_measured: n steps with the BulkQuantities row after each.

For SU(3) FP32 handles (FastTYMSolver, no current, masks or particles) each
step's kernel forms the per-site terms it can from what it loads (E^2 of the
new E, B^2 of its input links, the Gauss law of the state before it) and one
reduction follows the last step.  A twin handle on the same initial fields runs
opx_step(ctx, 1) + opx_reduce per step:
  - the fields after the run are bit-identical (the same update arithmetic);
  - the rows agree to FP32 rounding of the per-site terms (written tolerances);
  - a following step + reduce is bit-identical on both (the B^2 reuse holds).
Every other configuration, and nsteps = 1, is step + reduce itself: bit-identical.
"""
import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N
from tests.helpers import oracle_ic, fresh

pytestmark = pytest.mark.gpu


def vec(o):
    return np.array(list(o.e2) + list(o.b2) + [o.px, o.py, o.pz, o.gauss, o.rho2, o.e2_total, o.b2_total])


def twins(nc, dims, prec, reunit, seed=31, sigma=0.3, rho=False, kick=0.0):
    """Two handles on the same initial fields.  The oracle's initial E satisfies
    the Gauss law; kick adds Gaussian noise of that width to E (generator
    components) so that the Gauss-law term is far from zero."""
    g = fresh(oracle_ic(nc, dims, seed, sigma, sigma))
    hs = []
    e_kicked = None
    for _ in range(2):
        h = opx.Handle(nc, dims, a=g.a, dt=g.dt, g=g.g, precision=prec, reunit_every=reunit)
        h.upload(N.FIELD_U, g.U)
        h.upload(N.FIELD_E, g.E)
        if kick:
            if e_kicked is None:
                e = h.download(N.FIELD_E, layout=N.LAYOUT_GEN)
                e_kicked = e + np.random.default_rng(seed + 1).normal(0.0, kick, size=e.shape)
            h.upload(N.FIELD_E, e_kicked, layout=N.LAYOUT_GEN)
        if rho:
            r = np.random.default_rng(seed).normal(0.0, 0.05, size=h.V * h.ngen)
            h.upload(N.FIELD_RHO, r, layout=N.LAYOUT_GEN)
        h.initialize()
        hs.append(h)
    return hs


def loop(h, n):
    out = []
    for _ in range(n):
        h.step(1)
        out.append(h.reduce())
    return out


# FP32 rounding of the per-site terms: E^2 terms are identical per site (only the
# summation order differs), B^2 terms are products in another association, the
# Gauss-law terms are formed in another kernel (the same operations)
RTOL_E2 = 1e-6
RTOL_B2 = 3e-6
RTOL_GAUSS = 1e-5


@pytest.mark.parametrize("dims,reunit,rho,kick", [
    ((16, 16, 16), 4, False, 0.05),   # reunitarisation steps inside the run
    ((12, 10, 14), 0, True, 0.0),     # V = 1680: the last thread has one site; a static charge density
    ((24, 20, 16), 3, False, 0.05),
    ((3, 2, 5), 0, False, 0.05),      # V = 30: one warp, every thread with one site
])
def test_fused_rows_match_step_and_reduce(native, dims, reunit, rho, kick):
    a, b = twins(3, dims, N.OPX_F32, reunit, rho=rho, kick=kick)
    a.reduce(), b.reduce()
    n = 9
    ra = a.step_measured(n)
    rb = loop(b, n)
    assert a.steps_done == b.steps_done
    for f in (N.FIELD_U, N.FIELD_UNEXT, N.FIELD_E):
        assert np.array_equal(a.download(f), b.download(f)), f
    for oa, ob in zip(ra, rb):
        va, vb = vec(oa), vec(ob)
        scale = ob.e2_total + ob.b2_total
        np.testing.assert_allclose(va[0:3], vb[0:3], rtol=RTOL_E2, atol=0)
        np.testing.assert_allclose(va[3:6], vb[3:6], rtol=RTOL_B2, atol=0)
        np.testing.assert_allclose(va[6:9], vb[6:9], rtol=0, atol=RTOL_B2 * scale)
        np.testing.assert_allclose(va[9], vb[9], rtol=RTOL_GAUSS, atol=1e-9 * scale)
        assert va[10] == vb[10]  # rho^2: the same reduction
        np.testing.assert_allclose(va[11:], vb[11:], rtol=RTOL_B2, atol=0)
    # the Gauss law of these fields is far from zero (the kick or the charge
    # density), so the comparison above tests the Gauss term, not rounding noise
    assert rb[0].gauss > 1e-4 * (rb[0].e2_total + rb[0].b2_total)
    # a following step + reduce reuses B^2 and is bit-identical on both handles
    a.step(1)
    b.step(1)
    assert np.array_equal(vec(a.reduce()), vec(b.reduce()))


@pytest.mark.parametrize("nc,dims,prec,n", [
    (3, (8, 8, 8), N.OPX_F64, 5),
    (2, (10, 8, 12), N.OPX_F32, 5),
    (3, (12, 12, 12), N.OPX_F32, 1),   # one step: step + reduce
])
def test_other_forms_are_step_and_reduce(native, nc, dims, prec, n):
    a, b = twins(nc, dims, prec, 0)
    a.reduce(), b.reduce()
    ra = a.step_measured(n)
    rb = loop(b, n)
    for oa, ob in zip(ra, rb):
        assert np.array_equal(vec(oa), vec(ob))
    assert np.array_equal(a.download(N.FIELD_E), b.download(N.FIELD_E))


def test_masks_take_the_plain_path(native):
    a, b = twins(3, (12, 12, 12), N.OPX_F32, 0)
    ones = np.ones(a.V, dtype=np.uint8)
    a.set_evaluatable(ones)
    b.set_evaluatable(ones)
    ra = a.step_measured(4)
    rb = loop(b, 4)
    for oa, ob in zip(ra, rb):
        assert np.array_equal(vec(oa), vec(ob))


def test_invalid_arguments(native):
    a, _ = twins(3, (8, 8, 8), N.OPX_F32, 0)
    assert a.step_measured(0) == []
    with pytest.raises(opx.OpixiError):
        a.step_measured(-1)


def test_long_offsets_match(native, monkeypatch):
    """The measured step with 64-bit offsets (OPX_LONG_OFFSETS=1 at handle
    creation) against the 32-bit form: bit-identical fields and rows."""
    a, _ = twins(3, (12, 10, 14), N.OPX_F32, 4, kick=0.05)
    monkeypatch.setenv("OPX_LONG_OFFSETS", "1")
    b, _ = twins(3, (12, 10, 14), N.OPX_F32, 4, kick=0.05)
    monkeypatch.delenv("OPX_LONG_OFFSETS")
    ra, rb = a.step_measured(7), b.step_measured(7)
    for f in (N.FIELD_U, N.FIELD_UNEXT, N.FIELD_E):
        assert np.array_equal(a.download(f), b.download(f)), f
    for oa, ob in zip(ra, rb):
        assert np.array_equal(vec(oa), vec(ob))


def test_repeated_calls_continue_the_run(native):
    """Two calls of 4 and 5 steps give the rows of one call of 9 (the second
    call's first row takes its Gauss law and B^2 of Unext from its own kernels)."""
    a, b = twins(3, (16, 12, 10), N.OPX_F32, 3, kick=0.05)
    ra = a.step_measured(4) + a.step_measured(5)
    rb = b.step_measured(9)
    for f in (N.FIELD_U, N.FIELD_E):
        assert np.array_equal(a.download(f), b.download(f)), f
    for oa, ob in zip(ra, rb):
        va, vb = vec(oa), vec(ob)
        np.testing.assert_allclose(va, vb, rtol=RTOL_GAUSS, atol=RTOL_B2 * (ob.e2_total + ob.b2_total))


def test_simulation_run_uses_the_measured_loop(native, tmp_path):
    """Simulation.run with BulkQuantitiesInTime at every step as the only
    diagnostic hands the updates to opx_step_measured; its file has the rows of
    the step-by-step loop (Simulation.step while continues()) to FP32 rounding of
    the per-site terms, and the same number of rows (step 0 plus iterations + 1
    updates)."""
    from openpixi_gb300 import settings as S
    from openpixi_gb300.simulation import Simulation

    def deck(path):
        return f"""
simulationType: temporal yang-mills
gridStep: 1
couplingConstant: 1
numberOfDimensions: 3
numberOfColors: 3
gridCells: [12, 10, 16]
timeStep: 0.05
duration: 0.5
initialConditions:
  randomGaussian:
    - randomSeed: 11
      sigmaA: 0.2
      sigmaE: 0.2
output:
  bulkQuantitiesInTime:
    - path: {path}
      interval: 0.05
gpu:
  precision: f32
  reunitarizeEvery: 4
"""
    fa, fb = tmp_path / "a.txt", tmp_path / "b.txt"
    a = Simulation(S.settings_from_string(deck(fa)))
    b = Simulation(S.settings_from_string(deck(fb)))
    assert a._measured_loop()
    a.run()
    while b.continues():
        b.step()
    assert a.totalSimulationSteps == b.totalSimulationSteps == b.iterations + 1
    ra = [[float(v) for v in ln.split("\t")] for ln in fa.read_text().splitlines()[1:]]
    rb = [[float(v) for v in ln.split("\t")] for ln in fb.read_text().splitlines()[1:]]
    assert len(ra) == len(rb) == b.iterations + 2
    for x, y in zip(ra, rb):
        assert x[0] == y[0]
        scale = y[1] + y[2]
        np.testing.assert_allclose(x[1:3], y[1:3], rtol=RTOL_B2)
        np.testing.assert_allclose(x[3:6], y[3:6], rtol=0, atol=RTOL_B2 * scale)
        np.testing.assert_allclose(x[6], y[6], rtol=RTOL_GAUSS, atol=1e-9 * scale)
    for f in (N.FIELD_U, N.FIELD_E):
        assert np.array_equal(a.grid.handle.download(f), b.grid.handle.download(f))


def test_non_finite_fields_are_reported(native):
    """A NaN in E (planted on the host) ends the call with OPX_ERR_NUMERIC and
    the handle stays usable."""
    a, _ = twins(3, (8, 8, 8), N.OPX_F32, 0)
    e = a.download(N.FIELD_E, layout=N.LAYOUT_GEN)
    e.reshape(-1)[123] = np.nan
    a.upload(N.FIELD_E, e, layout=N.LAYOUT_GEN)
    with pytest.raises(N.OpixiError) as err:
        a.step_measured(3)
    assert err.value.code == N.OPX_ERR_NUMERIC
    a.upload(N.FIELD_E, np.zeros_like(e), layout=N.LAYOUT_GEN)
    a.upload(N.FIELD_U, identity_links(a))
    a.initialize()
    rows = a.step_measured(3)
    assert all(o.e2_total == 0.0 and o.b2_total == 0.0 for o in rows)


def identity_links(h):
    u = np.zeros((h.V, 3, 18))
    u[:, :, [0, 4, 8]] = 1.0  # re[0], re[4], re[8] of the row-major re[9], im[9] layout
    return u
