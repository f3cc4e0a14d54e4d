"""Batching form: independent lattices of uneven sizes advanced together (one
persistent launch of clusters of CTAs, or one launch per step over all events;
CUDA graph) against the same lattices stepped one by one through the
single-lattice path, and against the CPU oracle.

Tolerances: the batch and the single-lattice path run the same per-site
arithmetic, so their fields agree to 1e-12 (FP64) / 1e-6 (FP32) per link;
FP64 events agree with the oracle to 1e-10 per link.
"""
import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N
from tests.helpers import link_rel_err, field_rel_err

pytestmark = pytest.mark.gpu

DIMS = [(8, 8, 8), (12, 12, 12), (8, 16, 8), (16, 16, 16), (6, 6, 6), (16, 8, 24)]
SEEDS = [11, 12, 13, 14, 15, 16]


def single(nc, dims, seed, precision, steps, reunit=0, sigma=0.1):
    h = opx.Handle(nc, dims, dt=0.05, precision=precision, reunit_every=reunit)
    h.init_random(seed, sigma, sigma)
    h.gauss_project(1e-24 if precision == N.OPX_F32 else 1e-26)
    h.initialize()
    h.step(steps)
    return h


@pytest.mark.parametrize("nc,prec,tol", [(2, N.OPX_F64, 1e-12), (2, N.OPX_F32, 1e-5), (3, N.OPX_F32, 1e-5)])
@pytest.mark.parametrize("schedule", [None, (0, 128), (0, 256), (1, 128)])
def test_batch_matches_single_lattices(native, nc, prec, tol, schedule):
    """Both schedules (persistent clusters, the default; flat, cluster 0)."""
    reunit = 10 if prec == N.OPX_F32 else 0
    b = opx.Batch(nc, DIMS, dt=0.05, precision=prec, reunit_every=reunit)
    if schedule is not None:
        if nc == 3 and prec == N.OPX_F32 and schedule[1] == 256:
            with pytest.raises(N.OpixiError) as e:
                b.set_schedule(*schedule)
            assert e.value.code == N.OPX_ERR_UNSUPPORTED
            return
        b.set_schedule(*schedule)
    b.init_random(SEEDS, 0.1, 0.1, tol=1e-24 if prec == N.OPX_F32 else 1e-26)
    b.initialize()
    b.run(7)
    b.run(6)  # a second graph (other buffer parity)
    obs = b.reduce()
    for q, (d, s) in enumerate(zip(DIMS, SEEDS)):
        h = single(nc, d, s, prec, 13, reunit)
        assert link_rel_err(b.download(q, N.FIELD_U), h.download(N.FIELD_U)) <= tol
        assert field_rel_err(b.download(q, N.FIELD_E), h.download(N.FIELD_E)) <= tol
        o = h.reduce()
        assert abs(obs[q].e2_total + obs[q].b2_total - o.e2_total - o.b2_total) <= 1e-6 * (o.e2_total + o.b2_total)
        assert obs[q].gauss < (1e-10 if prec == N.OPX_F32 else 1e-20)


def test_batch_fp64_matches_oracle(native, orc):
    dims = [(6, 6, 6), (8, 4, 10)]
    b = opx.Batch(2, dims, dt=0.05, precision=N.OPX_F64)
    grids = []
    for q, d in enumerate(dims):
        g = orc.OracleGrid(2, d, dt=0.05)
        g.random_links(100 + q, 0.2)
        g.random_e(100 + q, 0.2)
        g.gauss_project()
        b.upload(q, N.FIELD_U, g.U)
        b.upload(q, N.FIELD_E, g.E)
        grids.append(g)
    b.initialize()
    b.run(10, use_graph=False)
    for q, g in enumerate(grids):
        sim = orc.OracleSimulation(g)
        sim.initialize()
        for _ in range(10):
            sim.step()
        assert link_rel_err(b.download(q, N.FIELD_U), g.U) <= 1e-10
        assert field_rel_err(b.download(q, N.FIELD_E), g.E) <= 1e-10


def test_autotune_restores_state_and_graph_equals_direct(native):
    b1 = opx.Batch(2, DIMS, precision=N.OPX_F32, reunit_every=10)
    b2 = opx.Batch(2, DIMS, precision=N.OPX_F32, reunit_every=10)
    for b in (b1, b2):
        b.init_random(SEEDS, 0.1, 0.1)
        b.initialize()
    c, blk = b1.autotune(steps=3)
    assert c in (0, 1, 2, 4, 8) and blk in (128, 256)
    b1.run(12, use_graph=True)
    b2.run(12, use_graph=False)
    for q in range(len(DIMS)):
        assert np.array_equal(b1.download(q, N.FIELD_U), b2.download(q, N.FIELD_U))
        assert np.array_equal(b1.download(q, N.FIELD_E), b2.download(q, N.FIELD_E))


def test_batch_errors(native):
    b = opx.Batch(2, DIMS[:2])
    with pytest.raises(N.OpixiError) as e:
        b.upload(5, N.FIELD_U, np.zeros((8, 3, 4)))
    assert e.value.code == N.OPX_ERR_INVALID
    with pytest.raises(N.OpixiError) as e:
        b.upload(0, N.FIELD_U, np.zeros(7))
    assert e.value.code == N.OPX_ERR_INVALID
