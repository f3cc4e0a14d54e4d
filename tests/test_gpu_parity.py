"""Parity of the CUDA leapfrog and reductions against the CPU FP64 oracle, through
the C ABI (libopixi_gpu.so).  Tolerances, stated per test:
  FP64: per-link relative error of U and E <= 1e-10 after the run; observables
        (energy, pressures) relative <= 1e-12; Gauss violation <= 1e-12.
  FP32: energy relative error vs the FP64 GPU run <= 1e-6.
"""
import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N
from tests.helpers import oracle_ic, fresh, link_rel_err, field_rel_err, to_gen

pytestmark = pytest.mark.gpu


def handle_from_oracle(g, precision=N.OPX_F64, reunit_every=0):
    h = opx.Handle(g.nc, g.dims, a=g.a, dt=g.dt, g=g.g, precision=precision, reunit_every=reunit_every)
    h.upload(N.FIELD_U, g.U)
    h.upload(N.FIELD_UNEXT, g.Unext)
    h.upload(N.FIELD_E, g.E)
    h.upload(N.FIELD_J, g.J)
    h.upload(N.FIELD_RHO, g.rho)
    return h


def bulk_vec(o):
    return np.array(list(o.e2) + list(o.b2) + [o.px, o.py, o.pz, o.gauss, o.rho2])


@pytest.mark.parametrize("nc,dims,steps,sigma", [
    (2, (32, 32, 32), 100, 0.1),   # the plain SU(2) FP64 workload: 32^3, dt = 0.05, 100 steps
    (3, (12, 12, 12), 30, 0.2),
    (2, (8, 12, 6), 40, 0.3),      # non-cubic
])
def test_leapfrog_fp64_matches_oracle(native, orc, nc, dims, steps, sigma):
    g = fresh(oracle_ic(nc, dims, 1234, sigma, sigma))
    h = handle_from_oracle(g)
    sim = orc.OracleSimulation(g)
    sim.initialize()
    h.initialize()
    e0 = None
    for k in range(steps):
        sim.step()
        h.step(1)
        if k % 10 == 9 or k == steps - 1:
            ob = g.bulk()
            od = h.reduce()
            ref = np.concatenate([ob[:9], ob[9:10]])
            dev = bulk_vec(od)[:10]
            et_ref, et_dev = ob[11] + ob[12], od.e2_total + od.b2_total
            if e0 is None:
                e0 = et_ref
            # energy (drift) matches the oracle's to 1e-12 relative
            assert abs(et_dev - et_ref) <= 1e-12 * abs(et_ref)
            assert np.all(np.abs(dev[:9] - ref[:9]) <= 1e-12 * np.abs(et_ref))
            # Gauss law stays satisfied
            assert od.gauss <= 1e-12
    U = h.download(N.FIELD_U)
    E = h.download(N.FIELD_E, layout=N.LAYOUT_GEN)
    assert link_rel_err(U, g.U) <= 1e-10
    assert field_rel_err(E, to_gen(orc, nc, g.E)) <= 1e-10
    Un = h.download(N.FIELD_UNEXT)
    assert link_rel_err(Un, g.Unext) <= 1e-10


def test_uneven_spacing_and_coupling(native, orc):
    g = orc.OracleGrid(2, (6, 8, 10), a=(1.0, 0.5, 2.0), dt=0.02, g=1.7)
    g.random_links(5, 0.2)
    g.random_e(5, 0.2)
    g.gauss_project()
    h = handle_from_oracle(g)
    sim = orc.OracleSimulation(g)
    sim.initialize()
    h.initialize()
    for _ in range(15):
        sim.step()
        h.step(1)
    assert link_rel_err(h.download(N.FIELD_U), g.U) <= 1e-10
    assert field_rel_err(h.download(N.FIELD_E), g.E) <= 1e-10
    ob, od = g.bulk(), h.reduce()
    assert abs(od.e2_total + od.b2_total - ob[11] - ob[12]) <= 1e-12 * (ob[11] + ob[12])


@pytest.mark.parametrize("nc", [2, 3])
def test_reductions_match_oracle(native, orc, nc):
    g = fresh(oracle_ic(nc, (8, 6, 10), 77, 0.4, 0.4))
    g.update_links()
    # non-zero charge density so that the Gauss and rho^2 columns are exercised
    rng = np.random.default_rng(3)
    rg = rng.normal(0, 0.1, (g.V, 3 if nc == 2 else 8))
    for x in range(g.V):
        g.rho[x] = orc.gen_to_alg(nc, rg[x])
    h = handle_from_oracle(g)
    ob, od = g.bulk(), h.reduce()
    assert np.allclose(bulk_vec(od), ob[:11], rtol=1e-12, atol=1e-15)
    assert np.allclose(h.energy_density(), g.energy_density(), rtol=1e-12, atol=1e-15)
    for d in range(3):
        assert np.allclose(h.projected_energy(d), g.projected_energy(d), rtol=1e-12, atol=1e-15)
    gf = h.gauss_field()
    gref = to_gen(orc, nc, g.gauss_field())
    assert np.abs(gf - gref).max() <= 1e-12 * max(1.0, np.abs(gref).max())


def test_evaluation_and_active_regions(native, orc):
    """Cell.isActive gates the update, Cell.isEvaluatable the reductions."""
    g = fresh(oracle_ic(2, (8, 8, 8), 21, 0.2, 0.2))
    act = np.zeros(g.V, np.uint8)
    ev = np.zeros(g.V, np.uint8)
    for x in range(g.V):
        p = (x // 64, (x // 8) % 8, x % 8)
        act[x] = 1 if 1 <= p[0] <= 6 else 0
        ev[x] = 1 if all(2 <= c <= 5 for c in p) else 0
    g.active[:] = act
    g.eval[:] = ev
    h = handle_from_oracle(g)
    h.set_active(act)
    h.set_evaluatable(ev)
    sim = orc.OracleSimulation(g)
    sim.initialize()
    h.initialize()
    for _ in range(6):
        sim.step()
        h.step(1)
    assert link_rel_err(h.download(N.FIELD_U), g.U) <= 1e-10
    assert np.allclose(bulk_vec(h.reduce()), g.bulk()[:11], rtol=1e-12, atol=1e-15)
    assert np.allclose(h.energy_density(), g.energy_density(), rtol=1e-12, atol=1e-15)


def test_fp32_su3_energy_error(native, orc):
    """Precision form: FP32 links/E with re-unitarisation every 10 steps against
    the FP64 GPU run: relative energy error <= 1e-6 after 100 steps."""
    g = fresh(oracle_ic(3, (16, 16, 16), 99, 0.2, 0.2))
    h64 = handle_from_oracle(g)
    h32 = handle_from_oracle(g, precision=N.OPX_F32, reunit_every=10)
    h64.initialize()
    h32.initialize()
    worst = 0.0
    for k in range(10):
        h64.step(10)
        h32.step(10)
        o64, o32 = h64.reduce(), h32.reduce()
        e64 = o64.e2_total + o64.b2_total
        e32 = o32.e2_total + o32.b2_total
        worst = max(worst, abs(e32 - e64) / e64)
        assert o32.gauss < 1e-10
    assert worst <= 1e-6, worst


def test_device_initial_conditions_match_oracle(native, orc):
    nc, dims = 3, (6, 6, 6)
    g = orc.OracleGrid(nc, dims)
    g.random_links(42, 0.2)
    g.random_e(42, 0.2)
    h = opx.Handle(nc, dims)
    h.init_random(42, 0.2, 0.2)
    assert link_rel_err(h.download(N.FIELD_U), g.U) <= 1e-13
    assert np.abs(h.download(N.FIELD_E, layout=N.LAYOUT_GEN) - to_gen(orc, nc, g.E)).max() <= 1e-14
    it, g2 = h.gauss_project(1e-26)
    assert g2 < 1e-26
    g.gauss_project(1e-26)
    assert field_rel_err(h.download(N.FIELD_E), g.E) <= 1e-8


def test_gauss_project_fp32_handle(native):
    h = opx.Handle(3, (16, 16, 16), precision=N.OPX_F32, reunit_every=10)
    h.init_random(7, 0.2, 0.2)
    it, g2 = h.gauss_project(1e-24)
    assert g2 < 1e-24
    h.initialize()
    h.step(20)
    assert h.reduce().gauss < 1e-10


def test_errors_are_status_codes(native):
    h = opx.Handle(2, (4, 4, 4))
    with pytest.raises(N.OpixiError) as e:
        h.upload(N.FIELD_U, np.zeros(7))
    assert e.value.code == N.OPX_ERR_INVALID
    with pytest.raises(N.OpixiError) as e:
        h.projected_energy(5)
    assert e.value.code == N.OPX_ERR_INVALID
    h32 = opx.Handle(2, (4, 4, 4), precision=N.OPX_F32)
    with pytest.raises(N.OpixiError) as e:
        h32.particles_upload(np.zeros((1, 3)), np.zeros((1, 3)), np.zeros((1, 3)), np.zeros((1, 3)),
                             np.zeros((1, 3)), np.zeros(1, np.int32))
    assert e.value.code == N.OPX_ERR_UNSUPPORTED
    # host-side fault injection: a NaN in E is reported by the reduction, the context stays usable
    E = np.zeros((64, 3, 3))
    E[5, 1, 2] = np.nan
    h.upload(N.FIELD_E, E)
    h.initialize()
    with pytest.raises(N.OpixiError) as e:
        h.reduce()
    assert e.value.code == N.OPX_ERR_NUMERIC
    h.upload(N.FIELD_E, np.zeros((64, 3, 3)))
    h.initialize()
    assert h.reduce().e2_total == 0.0


def _handle_env(g, scalar, **kw):
    import os
    if scalar:
        os.environ["OPX_ONE_SITE_FP32"] = "1"
    try:
        return handle_from_oracle(g, **kw)
    finally:
        os.environ.pop("OPX_ONE_SITE_FP32", None)


@pytest.mark.parametrize("dims,masked", [((16, 16, 16), False), ((7, 9, 11), True), ((5, 6, 33), False)])
def test_fp32_su3_pair_kernel(native, orc, dims, masked):
    """The SU(3) FP32 leapfrog that advances two sites per thread in paired FP32
    instructions against the one-site form and the FP64 run: links and E agree
    with the one-site form to FP32 rounding (2e-5 per link after 20 steps) and
    with FP64 to 1e-4; lattices whose volume is not a multiple of 64 and
    inactive cells take the masked lanes."""
    g = fresh(oracle_ic(3, dims, 5, 0.2, 0.2))
    if masked:
        act = (np.arange(g.V) % 5 != 3).astype(np.uint8)
        g.active[:] = act
    hp = _handle_env(g, False, precision=N.OPX_F32, reunit_every=10)
    hs = _handle_env(g, True, precision=N.OPX_F32, reunit_every=10)
    h64 = handle_from_oracle(g)
    if masked:
        for h in (hp, hs, h64):
            h.set_active(g.active)
    for h in (hp, hs, h64):
        h.initialize()
        h.step(20)
    up, us, u64 = (h.download(N.FIELD_U) for h in (hp, hs, h64))
    ep, es, e64 = (h.download(N.FIELD_E) for h in (hp, hs, h64))
    assert link_rel_err(up, us) <= 2e-5
    assert field_rel_err(ep, es) <= 2e-5
    assert link_rel_err(up, u64) <= 1e-4
    assert field_rel_err(ep, e64) <= 1e-4
    if masked:
        off = g.active == 0
        U0 = g.U
        assert np.array_equal(up[off], U0[off].astype(np.float32).astype(np.float64)) or \
            np.abs(up[off] - U0[off]).max() < 1e-6


@pytest.mark.parametrize("dims", [(16, 16, 16), (7, 9, 11)])
def test_fp32_su3_pair_reduction(native, orc, dims):
    """The paired SU(3) FP32 BulkQuantities pass against the one-site pass on the
    same FP32 fields, with an evaluation mask and a charge density: every column
    within 1e-6 relative (the per-site values are formed in FP32 both ways)."""
    g = fresh(oracle_ic(3, dims, 8, 0.3, 0.3))
    rng = np.random.default_rng(4)
    g.rho[...] = rng.normal(0, 0.1, g.rho.shape)
    ev = (np.arange(g.V) % 7 != 2).astype(np.uint8)
    hp = _handle_env(g, False, precision=N.OPX_F32, reunit_every=10)
    hs = _handle_env(g, True, precision=N.OPX_F32, reunit_every=10)
    for h in (hp, hs):
        h.set_evaluatable(ev)
        h.initialize()
        h.step(3)
    a, b = bulk_vec(hp.reduce()), bulk_vec(hs.reduce())
    assert np.all(np.abs(a - b) <= 1e-6 * np.abs(b) + 1e-12), (a, b)


def test_projected_poynting_matches_oracle(native, orc):
    """ProjectedEnergyDensity Poynting rows (SU(2)) against the oracle on a
    lattice with uneven spacings, every direction: 1e-12 of the largest
    row value; SU(3) handles report OPX_ERR_UNSUPPORTED (the reference throws)."""
    g = fresh(oracle_ic(2, (8, 6, 10), 31, 0.4, 0.3, dt=0.1, a=(1.0, 0.9, 1.2)))
    h = handle_from_oracle(g)
    sim = orc.OracleSimulation(g)
    sim.initialize()
    h.initialize()
    for _ in range(3):
        sim.step()
        h.step(1)
    for d in range(3):
        ref = g.projected_poynting(d)
        got = h.projected_poynting(d)
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), d
    h3 = opx.Handle(3, (4, 4, 4))
    with pytest.raises(opx.OpixiError):
        h3.projected_poynting(0)


@pytest.mark.parametrize("nc,dims", [(2, (1, 8, 8)), (2, (2, 1, 16)), (3, (3, 4, 1)), (2, (1, 1, 1))])
def test_degenerate_lattices(native, orc, nc, dims):
    """Directions with one or two cells (the periodic neighbour is the cell
    itself or its only other cell): FP64 leapfrog and reductions against the oracle."""
    g = fresh(oracle_ic(nc, dims, 17, 0.3, 0.3))
    h = handle_from_oracle(g)
    sim = orc.OracleSimulation(g)
    sim.initialize()
    h.initialize()
    for _ in range(5):
        sim.step()
        h.step(1)
    assert link_rel_err(h.download(N.FIELD_U), g.U) <= 1e-10
    assert field_rel_err(h.download(N.FIELD_E), g.E) <= 1e-10
    assert np.allclose(bulk_vec(h.reduce()), g.bulk()[:11], rtol=1e-10, atol=1e-14)


def test_empty_particle_list_and_oversized_lattice(native):
    """An empty particle list gives zero charge and current; a lattice beyond
    the 32-bit particle-cell keys is refused with a status code and the device
    stays usable."""
    h = opx.Handle(2, (8, 8, 8), dt=0.5)
    z3 = np.zeros((0, 3))
    h.particles_upload(z3, z3, z3, z3, z3, np.zeros(0, np.int32))
    h.initialize()
    h.step(2)
    assert np.all(h.download(N.FIELD_RHO) == 0) and np.all(h.download(N.FIELD_J) == 0)
    with pytest.raises(opx.OpixiError) as err:
        opx.Handle(3, (4096, 4096, 2048), precision=N.OPX_F64)
    assert err.value.code in (N.OPX_ERR_INVALID, N.OPX_ERR_NOMEM)
    h2 = opx.Handle(2, (8, 8, 8))  # the device is still usable
    h2.initialize()


@pytest.mark.parametrize("nc,prec", [(3, N.OPX_F32), (3, N.OPX_F64), (2, N.OPX_F32), (2, N.OPX_F64)])
def test_long_offsets_match(native, nc, prec):
    """The leapfrog and reduction kernels with 64-bit site and element offsets
    (the forms lattices too large for 32-bit offsets take; OPX_LONG_OFFSETS=1
    selects them at any size) against the 32-bit forms on a small lattice:
    bit-identical links, E and observables, with a current and (FP32) with
    re-unitarisation steps."""
    import os
    g = fresh(oracle_ic(nc, (7, 9, 11), 21, 0.2, 0.2))
    rng = np.random.default_rng(8)
    g.J[...] = rng.normal(0, 0.02, g.J.shape)
    ru = 4 if prec == N.OPX_F32 else 0
    ha = handle_from_oracle(g, precision=prec, reunit_every=ru)
    os.environ["OPX_LONG_OFFSETS"] = "1"
    try:
        hb = handle_from_oracle(g, precision=prec, reunit_every=ru)
    finally:
        os.environ.pop("OPX_LONG_OFFSETS", None)
    for h in (ha, hb):
        h.initialize()
        h.step(9)
    for f in (N.FIELD_U, N.FIELD_UNEXT, N.FIELD_E):
        assert np.array_equal(ha.download(f), hb.download(f)), f
    assert np.array_equal(bulk_vec(ha.reduce()), bulk_vec(hb.reduce()))
    ha.step(1)
    hb.step(1)
    assert np.array_equal(bulk_vec(ha.reduce()), bulk_vec(hb.reduce()))
