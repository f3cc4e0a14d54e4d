"""CPU checks of the CGC oracle (MV model, light-cone Poisson solver, particle creator).

The reference ships no test for these classes, so the oracle is pinned by
published values of java.util.Random (the generator the MV charges come
from) and by the properties the reference's construction guarantees:
the 2D Poisson equation holds sheet by sheet, refinement moves charge only
within a cell, and the particles' charge cancels the Gauss violation of the
fields after Simulation.initialize.
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def cgc(orc):
    from oracle import cgc as m
    return m


def test_java_random_known_values(cgc):
    # values printed by java.util.Random as documented in the Java SE API
    assert cgc.java_random(42, 2, 1)[0] == -1170105035.0
    assert cgc.java_random(42, 1, 1)[0] == 0.7275636800328681
    assert cgc.java_random(42, 0, 1)[0] == 1.1419053154730547
    assert cgc.java_random(0, 0, 1)[0] == 0.8025330637390305
    # nextGaussian draws pairs: the second of a pair comes from the cache
    g = cgc.java_random(7, 0, 6)
    assert len(set(g.tolist())) == 6


def test_poisson2d_solves_lattice_laplacian(cgc):
    rng = np.random.default_rng(1)
    dims = (4, 8, 6)
    rho = rng.normal(size=int(np.prod(dims)))
    phi = cgc.poisson2d(rho, dims, aT=0.7).reshape(dims)
    lap = sum(np.roll(phi, 1, ax) + np.roll(phi, -1, ax) - 2 * phi for ax in (1, 2)) / 0.7 ** 2
    r = rho.reshape(dims)
    r = r - r.mean(axis=(1, 2), keepdims=True)
    assert np.abs(-lap - r).max() < 1e-13


def test_regulation_removes_kt_zero_modes(cgc):
    rng = np.random.default_rng(2)
    dims = (8, 8, 8)
    r = cgc.regulate(rng.normal(size=512), dims, uvt=4.44, long_width=0.0, ir=0.0, aT=1.0, aL=1.0).reshape(dims)
    # every kT = 0 mode is cut, so each longitudinal sheet sums to zero
    assert np.abs(r.sum(axis=(1, 2))).max() < 1e-12
    # with no UV cut, no IR mass and no longitudinal smoothing only the kT = 0 modes go
    x = rng.normal(size=512).reshape(dims)
    y = cgc.regulate(x.reshape(-1), dims, uvt=10.0, long_width=0.0, ir=0.0, aT=1.0, aL=1.0).reshape(dims)
    assert np.allclose(y, x - x.mean(axis=(1, 2), keepdims=True), atol=1e-13)


@pytest.mark.parametrize("nc", [2, 3])
def test_single_nucleus_gauss_law_after_initialize(orc, cgc, nc):
    g = orc.OracleGrid(nc, (32, 6, 6), dt=0.5)
    P, info = cgc.cgc_mv(g, [cgc.MVNucleus(orientation=1, location=16.0, width=1.5, mu=0.5, seed=11)])
    ppc = 2
    assert P.n % (36 * ppc) == 0
    # cell sums of the refined charges equal the Gauss violation (refinement is cell-local)
    gauss = info[0]["gauss"]
    rho = np.zeros_like(gauss)
    cells = np.rint(P.pos0[:, 0]).astype(int) * 36 + np.rint(P.pos0[:, 1]).astype(int) * 6 + np.rint(P.pos0[:, 2]).astype(int)
    np.add.at(rho, cells, P.Q0)
    z = np.arange(g.V) // 36
    zs = np.unique(np.rint(P.pos0[:, 0]).astype(int))
    inside = np.isin(z, zs)
    assert np.abs(rho[inside] - gauss[inside]).max() < 1e-12 * np.abs(gauss).max()
    sim = orc.OracleSimulation(g, P)
    sim.initialize()
    gmax = np.abs(g.rho).max()
    assert np.abs(g.gauss_field()).max() < 1e-8 * gmax
    for _ in range(10):
        sim.step()
    assert np.abs(g.gauss_field()).max() < 1e-8 * gmax


def test_particle_layout(orc, cgc):
    g = orc.OracleGrid(2, (24, 4, 4), dt=0.25)
    P, _ = cgc.cgc_mv(g, [cgc.MVNucleus(orientation=-1, location=12.0, width=1.0, mu=0.5, seed=3)])
    ppc = 4
    nz = P.n // (16 * ppc)
    assert P.n == nz * 16 * ppc
    # particle k = ((z - zStart) * ntr + t) * ppc + j
    k = np.arange(P.n)
    j = k % ppc
    t = (k // ppc) % 16
    z0 = int(np.rint(P.pos0[0, 0] + 0.5 * 1.0))
    assert np.allclose(P.pos0[:, 0], (z0 + k // (ppc * 16)) + (j - ppc // 2) / ppc + 1e-11, atol=1e-12)
    assert np.array_equal(P.pos0[:, 1], np.floor(P.pos0[:, 1]) + 1e-11) or np.allclose(P.pos0[:, 1], t // 4 + 1e-11)
    assert np.allclose(P.pos1[:, 0] - P.pos0[:, 0], -0.25)
    assert np.all(P.vel[:, 0] == -1.0) and np.all(P.vel[:, 1:] == 0.0)


def test_super_particles_subdivision_invariant_and_gauss(orc, cgc):
    """LightConeNGPSuperParticleCreator + CGCSuperParticleInterpolationNGP: the
    result depends on how the particle block is split among threads
    (numberOfThreads) only through the summation order (1e-14 here), the Gauss
    law holds through the run, and the physics agrees with the NGP particles of
    the same nuclei."""
    nuclei = [cgc.MVNucleus(orientation=1, location=12.0, width=1.5, mu=0.5, seed=3),
              cgc.MVNucleus(orientation=-1, location=28.0, width=1.5, mu=0.5, seed=4)]
    runs = []
    for nt in (1, 3, 7):
        g = orc.OracleGrid(2, (40, 6, 6), dt=0.5)
        groups, _ = cgc.cgc_mv_super(g, nuclei)
        sim = cgc.OracleSuperSimulation(g, groups, nthreads=nt)
        sim.initialize()
        g0 = np.abs(g.gauss_field()).max()
        for _ in range(12):
            sim.step()
        assert np.abs(g.gauss_field()).max() <= 1.01 * g0 + 1e-12
        runs.append((g.U.copy(), g.E.copy(), g.J.copy()))
    for r in runs[1:]:
        for a, b in zip(r, runs[0]):
            assert np.abs(a - b).max() <= 1e-14 * np.abs(b).max()
    g2 = orc.OracleGrid(2, (40, 6, 6), dt=0.5)
    P, _ = cgc.cgc_mv(g2, nuclei)
    s2 = orc.OracleSimulation(g2, P)
    s2.initialize()
    for _ in range(12):
        s2.step()
    assert np.abs(runs[0][0] - g2.U).max() < 1e-3


# ---- WilsonLineObservables (physics/initial/CGC/WilsonLineObservables.java) ----

def _dipole_numpy(vt, nc, n1, n2, a1, a2):
    """Independent restatement of computeDipole (:67-131) with numpy."""
    total = n1 * n2
    nb = int(np.sqrt(total)) // 2
    ds = min(n1 * a1, n2 * a2) * 0.5 / nb
    pos = np.stack([np.arange(total) // n2, np.arange(total) % n2], 1)
    d = np.abs(pos[:, None, :] - pos[None, :, :]).astype(float)
    for k, n in enumerate((n1, n2)):
        d[..., k] = np.where(d[..., k] > n // 2, d[..., k] - n, d[..., k])
    dist = np.sqrt(d[..., 0] ** 2 * a1 * a1 + d[..., 1] ** 2 * a2 * a2)
    b = (dist / ds).astype(int)
    if nc == 2:
        tr = 2.0 * vt @ vt.T
    else:
        tr = vt @ vt.T  # sum of re*re + im*im over the 9 entries = Re tr(V1 V2^dagger)
    out = np.array([tr[b == k].mean() if np.any(b == k) else np.nan for k in range(nb)])
    return out, ds


def _random_vt(nc, n, seed):
    rng = np.random.default_rng(seed)
    if nc == 2:
        q = rng.normal(size=(n, 4))
        return q / np.linalg.norm(q, axis=1, keepdims=True)
    from scipy.stats import unitary_group
    out = np.empty((n, 18))
    for i in range(n):
        u = unitary_group.rvs(3, random_state=seed * 1000 + i)
        u = u / np.linalg.det(u) ** (1.0 / 3.0)
        out[i, :9] = u.real.reshape(-1)
        out[i, 9:] = u.imag.reshape(-1)
    return out


@pytest.mark.parametrize("nc,n1,n2,a1,a2", [(2, 8, 6, 1.0, 1.0), (2, 7, 9, 0.8, 1.3), (3, 6, 6, 1.0, 1.0)])
def test_wilson_dipole_matches_numpy(orc, nc, n1, n2, a1, a2):
    from oracle import cgc
    vt = _random_vt(nc, n1 * n2, 3)
    got, ds = cgc.wilson_dipole(vt, nc, n1, n2, a1, a2)
    ref, ds_ref = _dipole_numpy(vt, nc, n1, n2, a1, a2)
    assert ds == ds_ref
    assert np.allclose(got, ref, rtol=1e-13, atol=1e-13, equal_nan=True)


def test_wilson_observables_known_answers(orc):
    """Identity Wilson lines: tadpole N_c, every occupied dipole bin N_c; a
    global rotation V -> g V leaves the dipole unchanged."""
    from oracle import cgc
    for nc, ng in ((2, 4), (3, 18)):
        vt = np.zeros((64, ng))
        vt[:, 0] = 1.0
        if nc == 3:
            vt[:, 4] = vt[:, 8] = 1.0
        assert cgc.wilson_tadpole(vt, nc) == float(nc)
        d, _ = cgc.wilson_dipole(vt, nc, 8, 8)
        assert np.all(d[np.isfinite(d)] == float(nc))
    vt = _random_vt(2, 48, 9)
    g = _random_vt(2, 1, 10)[0]
    # quaternion product g * V (SU2GroupElement.mult)
    def qmul(x, a):
        return np.stack([x[0] * a[:, 0] - x[1] * a[:, 1] - x[2] * a[:, 2] - x[3] * a[:, 3],
                         x[0] * a[:, 1] + x[1] * a[:, 0] - x[2] * a[:, 3] + x[3] * a[:, 2],
                         x[0] * a[:, 2] + x[2] * a[:, 0] - x[3] * a[:, 1] + x[1] * a[:, 3],
                         x[0] * a[:, 3] + x[3] * a[:, 0] - x[1] * a[:, 2] + x[2] * a[:, 1]], 1)
    d0, _ = cgc.wilson_dipole(vt, 2, 8, 6)
    d1, _ = cgc.wilson_dipole(qmul(g, vt), 2, 8, 6)
    assert np.allclose(d0, d1, rtol=1e-13, atol=1e-13, equal_nan=True)
