"""Reuse of B^2 between per-step reductions.

opx_reduce after opx_step(ctx, 1), which followed an opx_reduce, takes B^2 of U
from the previous reduction's B^2 of Unext (the same links after the storeFields
swap) and sums only the plaquettes of Unext.  Read-only entry points in between
(downloads, diagnostics, synchronisation) keep the reuse; any entry point that
may change the fields or the masks turns it off.  The observables must be
bit-identical to a full recomputation: a twin handle on the same initial fields
sets an all-true evaluation mask between step and reduce (no change to the
sums, but a mask call), which disables the reuse.  Every run is also checked
against the CPU FP64 oracle once.
"""
import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N
from tests.helpers import oracle_ic, fresh

pytestmark = pytest.mark.gpu


def vec(o):
    return np.array(list(o.e2) + list(o.b2) + [o.px, o.py, o.pz, o.gauss, o.rho2, o.e2_total, o.b2_total])


def twin_handles(nc, dims, prec, reunit, seed, sigma, implicit=False):
    g = fresh(oracle_ic(nc, dims, seed, sigma, sigma))
    hs = []
    for _ in range(2):
        h = opx.Handle(nc, dims, a=g.a, dt=g.dt, g=g.g, precision=prec, reunit_every=reunit)
        h.upload(N.FIELD_U, g.U)
        h.upload(N.FIELD_E, g.E)
        if implicit:
            h.set_field_solver(N.SOLVER_IMPLICIT, 3, 0.0)
        h.initialize()
        hs.append(h)
    return g, hs


@pytest.mark.parametrize("nc,dims,prec,reunit,implicit", [
    (2, (16, 12, 10), N.OPX_F64, 0, False),
    (3, (12, 10, 14), N.OPX_F64, 0, False),
    (3, (16, 16, 16), N.OPX_F32, 4, False),   # the paired SU(3) FP32 reduction, reunitarisation on
    (2, (10, 8, 12), N.OPX_F32, 0, False),
    (2, (8, 8, 8), N.OPX_F64, 0, True),       # ImplicitTYMSolver steps
])
def test_reuse_bit_identical(native, orc, nc, dims, prec, reunit, implicit):
    g, (a, b) = twin_handles(nc, dims, prec, reunit, 77, 0.25, implicit)
    ra, rb = [a.reduce()], [b.reduce()]
    ones = np.ones(a.V, dtype=np.uint8)
    for k in range(12):
        a.step(1)
        if k % 3 == 1:  # read-only calls between step and reduce keep the reuse
            a.energy_density()
            a.download(N.FIELD_U)
            a.synchronize()
        ra.append(a.reduce())
        b.step(1)
        b.set_evaluatable(ones)  # a mask call: recompute everything
        rb.append(b.reduce())
    for oa, ob in zip(ra, rb):
        assert np.array_equal(vec(oa), vec(ob)), (vec(oa), vec(ob))
    if prec == N.OPX_F64 and not implicit:
        sim = orc.OracleSimulation(g)
        sim.initialize()
        for _ in range(12):
            sim.step()
        ref = g.bulk()
        got = vec(ra[-1])
        et = ref[11] + ref[12]
        assert abs(got[11] + got[12] - et) <= 1e-12 * abs(et)
        assert np.all(np.abs(got[:9] - ref[:9]) <= 1e-12 * abs(et))


def test_reuse_disabled_by_other_calls(native):
    """step(1), then an upload of other links, then reduce: B^2 of U must come
    from the uploaded links, not from the previous reduction."""
    rng = np.random.default_rng(5)
    _, (a, b) = twin_handles(2, (12, 12, 12), N.OPX_F64, 0, 91, 0.3)
    a.reduce()
    b.reduce()
    a.step(1)
    b.step(1)
    U = a.download(N.FIELD_U)
    q = U + rng.normal(0, 0.05, U.shape)
    q /= np.linalg.norm(q, axis=-1, keepdims=True)
    a.upload(N.FIELD_U, q)
    b.upload(N.FIELD_U, q)
    b.set_evaluatable(np.ones(b.V, dtype=np.uint8))
    oa, ob = a.reduce(), b.reduce()
    assert np.array_equal(vec(oa), vec(ob))
    # and the reuse after a multi-step call stays off as well
    a.step(3)
    b.step(3)
    b.set_evaluatable(np.ones(b.V, dtype=np.uint8))
    assert np.array_equal(vec(a.reduce()), vec(b.reduce()))


@pytest.mark.parametrize("nc,dims,prec", [(2, (12, 8, 10), N.OPX_F64), (3, (8, 10, 6), N.OPX_F32)])
def test_projected_energy_reuse_bit_identical(native, orc, nc, dims, prec):
    """ProjectedEnergyDensity after one step takes the magnetic rows of U from the
    previous call's Unext rows (per direction), interleaved with BulkQuantities
    as a per-step diagnostics loop does; bit-identical to the recomputing twin,
    and the FP64 rows match the oracle."""
    g, (a, b) = twin_handles(nc, dims, prec, 0, 5, 0.3)
    ones = np.ones(a.V, dtype=np.uint8)
    for h in (a, b):
        h.reduce()
        h.projected_energy(0)
        h.projected_energy(2)
    for k in range(6):
        a.step(1)
        b.step(1)
        b.set_evaluatable(ones)
        oa, ob = a.reduce(), b.reduce()
        assert np.array_equal(vec(oa), vec(ob))
        for d in (0, 2):
            pa, pb = a.projected_energy(d), b.projected_energy(d)
            assert np.array_equal(pa, pb), (k, d)
    if prec == N.OPX_F64:
        sim = orc.OracleSimulation(g)
        sim.initialize()
        for _ in range(6):
            sim.step()
        for d in (0, 2):
            ref = g.projected_energy(d)
            got = a.projected_energy(d)
            assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), d


@pytest.mark.parametrize("nc,dims,prec,masked", [
    (2, (12, 8, 10), N.OPX_F64, False),
    (2, (10, 9, 8), N.OPX_F64, True),
    (3, (8, 10, 6), N.OPX_F64, False),
    (2, (8, 12, 10), N.OPX_F32, False),
])
def test_projected_energy_from_reduction_sites(native, nc, dims, prec, masked):
    """ProjectedEnergyDensity right after opx_reduce on the same state reads the
    per-site B^2 of Unext that the BulkQuantities pass left (no plaquettes
    formed again); a twin that calls it before the reduction forms them.  Rows
    and observables bit-identical, with and without an evaluation region."""
    g, (a, b) = twin_handles(nc, dims, prec, 0, 9, 0.3)
    if masked:
        m = (np.arange(a.V) % 7 != 2).astype(np.uint8)
        a.set_evaluatable(m)
        b.set_evaluatable(m)
    for k in range(5):
        oa = a.reduce()
        pa = [a.projected_energy(d) for d in (0, 1)]
        pb = [b.projected_energy(d) for d in (0, 1)]
        ob = b.reduce()
        assert np.array_equal(vec(oa), vec(ob)), k
        for x, y in zip(pa, pb):
            assert np.array_equal(x, y), k
        a.step(1)
        b.step(1)
