"""CPIC (NGP) phases on the GPU against the sequential oracle, through the C ABI.

From an identical state, one step of the particle phases is bit-exact: particle
positions and cells, parallel-transported charges, and the rho / J deposits
(CGCParticleInterpolationNGP + CGCParticleSolver order).  Over a coupled run
the particle positions stay bit-exact; charges and fields agree to 1e-10
(the links they are transported with differ only by rounding).
"""
import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N
from tests.helpers import oracle_ic, fresh, link_rel_err, field_rel_err, to_gen

pytestmark = pytest.mark.gpu


def random_particles(orc, nc, dims, n, seed, dt=0.5):
    rng = np.random.default_rng(seed)
    P = orc.OracleParticles(nc, n)
    P.dir[:] = rng.choice([0, 0, 0, 1, 2], n)
    sign = rng.choice([-1.0, 1.0], n)
    for k in range(n):
        P.vel[k, P.dir[k]] = sign[k]
    P.pos0[:] = rng.uniform(0, 1, (n, 3)) * np.array(dims)
    # a quarter of the particles start exactly on half-integer positions (rint ties)
    ties = rng.random(n) < 0.25
    P.pos0[ties] = np.floor(P.pos0[ties]) + 0.5
    P.pos1[:] = P.pos0 - P.vel * dt
    gen = rng.normal(0, 0.3, (2, n, 3 if nc == 2 else 8))
    for k in range(n):
        P.Q0[k] = orc.gen_to_alg(nc, gen[0, k])
        P.Q1[k] = orc.gen_to_alg(nc, gen[1, k])
    return P


def upload_particles(h, P):
    h.particles_upload(P.pos0, P.pos1, P.vel, P.Q0, P.Q1, P.dir)


def oracle_phases(orc, g, P, reassign):
    import ctypes as C
    from oracle import lib, _p
    L = lib()
    if reassign:
        L.orc_cpic_reassign(g.nc, C.c_long(P.n), _p(P.pos0), _p(P.pos1), _p(P.Q0), _p(P.Q1))
    sim = orc.OracleSimulation(g, P)
    sim._cpic_phases()


def same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


@pytest.mark.parametrize("nc", [2, 3])
@pytest.mark.parametrize("reassign", [False, True])
def test_one_step_bit_exact(native, orc, nc, reassign):
    dims = (16, 8, 8)
    g = orc.OracleGrid(nc, dims, dt=0.5)
    g.random_links(3, 0.5)
    g.Unext[...] = g.U  # the transporters are read from Unext
    g.random_links(4, 0.5)
    g.U, g.Unext = g.Unext.copy(), g.U.copy()
    P = random_particles(orc, nc, dims, 4000, seed=10 + nc)
    h = opx.Handle(nc, dims, dt=0.5)
    h.upload(N.FIELD_UNEXT, g.Unext)
    upload_particles(h, P)
    h.cpic_phases(reassign=reassign)
    oracle_phases(orc, g, P, reassign)
    d = h.particles_download()
    for k in ("pos0", "pos1", "Q0", "Q1"):
        assert same_bits(d[k], getattr(P, k)), k
    rho = h.download(N.FIELD_RHO, layout=N.LAYOUT_GEN)
    J = h.download(N.FIELD_J, layout=N.LAYOUT_GEN)
    assert same_bits(rho, to_gen(orc, nc, g.rho))
    assert same_bits(J, to_gen(orc, nc, g.J))
    assert np.abs(J).max() > 0 and np.abs(rho).max() > 0


def test_deposit_order_with_crowded_cells(native, orc):
    """Many particles in few cells: each cell's sum is taken in particle order."""
    nc, dims = 2, (4, 2, 2)
    g = orc.OracleGrid(nc, dims, dt=0.5)
    g.random_links(8, 0.7)
    P = random_particles(orc, nc, dims, 5000, seed=1)
    rng = np.random.default_rng(2)
    P.Q0 *= 10.0 ** rng.integers(-8, 8, (P.n, 1))   # wide magnitudes: order matters
    h = opx.Handle(nc, dims, dt=0.5)
    h.upload(N.FIELD_UNEXT, g.Unext)
    upload_particles(h, P)
    h.cpic_phases(reassign=False)
    oracle_phases(orc, g, P, False)
    assert same_bits(h.download(N.FIELD_RHO), g.rho)
    assert same_bits(h.download(N.FIELD_J), g.J)


def test_coupled_run(native, orc):
    """storeFields + updateGrid + particle phases over 40 steps (SU(2), dt = 0.5)."""
    nc, dims = 2, (24, 8, 8)
    g = orc.OracleGrid(nc, dims, dt=0.5)
    g.random_links(12, 0.1)
    P = random_particles(orc, nc, dims, 3000, seed=5)
    h = opx.Handle(nc, dims, dt=0.5)
    h.upload(N.FIELD_U, g.U)
    upload_particles(h, P)
    sim = orc.OracleSimulation(g, P)
    sim.initialize()
    h.initialize()
    for _ in range(40):
        sim.step()
        h.step(1)
    d = h.particles_download()
    assert same_bits(d["pos0"], P.pos0) and same_bits(d["pos1"], P.pos1)
    assert field_rel_err(d["Q0"], P.Q0) <= 1e-10
    assert field_rel_err(h.download(N.FIELD_E), g.E) <= 1e-10
    assert link_rel_err(h.download(N.FIELD_U), g.U) <= 1e-10
    assert field_rel_err(h.download(N.FIELD_RHO), g.rho) <= 1e-10
    ob, od = g.bulk(), h.reduce()
    assert abs(od.e2_total + od.b2_total - ob[11] - ob[12]) <= 1e-10 * (ob[11] + ob[12])
