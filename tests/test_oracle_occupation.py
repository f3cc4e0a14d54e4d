"""CPU checks of the Coulomb-gauge / occupation-number oracle (SU(2)).

Pins: the reference's CoulombGaugeTest known answers (iteration counts on a
2x2x2 lattice: a trivial configuration converges in 1 iteration, an abelian
gauge transformation in exactly 2, a non-abelian one in more than 2, each to
the accuracy goal), gauge invariance of the occupation numbers' input (the
Coulomb-gauge result does not depend on a prior random gauge transformation
beyond the residual), and the energy from the occupation numbers against the
field energy for weak fields."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def occ(orc):
    from oracle import occupation as m
    return m


def gauge_transform(orc, g, psi):
    """GaugeTransformation with g(x) = getLink(-psi(x)) applied to U, Unext, E."""
    from oracle import lib, _p
    L = lib()
    L.orc_coulomb_apply.argtypes = [C.c_void_p] * 5
    L.orc_coulomb_apply(g.pp, _p(np.ascontiguousarray(psi)), _p(g.U), _p(g.Unext), _p(g.E))


@pytest.mark.parametrize("f1,f2,expect", [((0, 0, 0), (0, 0, 0), "1"), ((.1, 0, 0), (0, 0, 0), "2"),
                                          ((.1, 0, 0), (0, .1, 0), ">2")])
def test_coulomb_gauge_known_answers(orc, occ, f1, f2, expect):
    # CoulombGaugeTest.testForSU2Fields: 2x2x2 trivial field, g at sites 0 and 1
    g = orc.OracleGrid(2, (2, 2, 2), dt=0.1)
    psi = np.zeros((3, 8))
    psi[:, 0] = -np.array(f1)
    psi[:, 1] = -np.array(f2)
    gauge_transform(orc, g, psi)
    conv = occ.coulomb_gauge(g)
    assert conv[-1] < 1e-18
    if expect == "1":
        assert len(conv) == 1
    elif expect == "2":
        assert len(conv) == 2
    else:
        assert len(conv) > 2


def test_occupation_energy_weak_field(orc, occ):
    """For weak fields the energy from the occupation numbers equals the
    field energy 1/2 <E^2 + B^2> in physical units up to O(field^4) corrections."""
    g = orc.OracleGrid(2, (8, 8, 8), dt=0.05)
    g.random_links(5, 0.02)
    g.random_e(5, 0.02)
    g.gauss_project(tol_g2=1e-28)
    sim = orc.OracleSimulation(g)
    sim.initialize()
    n, energy, conv = occ.occupation_numbers(g)
    assert conv[-1] < 1e-18
    b = g.bulk()
    field_energy = 0.5 * (b[11] + b[12])
    assert abs(energy - field_energy) <= 0.05 * field_energy, (energy, field_energy)
    assert np.all(n.sum(axis=1) > -1e-12 * n.max())


def test_occupation_gauge_invariant(orc, occ):
    """A random gauge transformation before the measurement changes the
    colour-summed occupation numbers and the energy only at the level of the
    Coulomb-gauge residual (the Coulomb gauge leaves a global colour rotation,
    which mixes the colour components)."""
    g = orc.OracleGrid(2, (6, 6, 6), dt=0.05)
    g.random_links(7, 0.1)
    g.random_e(7, 0.1)
    g.update_links()
    n0, e0, _ = occ.occupation_numbers(g)
    rng = np.random.default_rng(3)
    gauge_transform(orc, g, rng.normal(0, 0.2, (3, g.V)))
    n1, e1, _ = occ.occupation_numbers(g)
    assert abs(e1 - e0) <= 1e-6 * e0
    s0, s1 = n0.sum(axis=1), n1.sum(axis=1)
    assert np.abs(s1 - s0).max() <= 1e-5 * np.abs(s0).max()


def test_mirror_roundtrip_and_windows(orc):
    """MirroredGrid then UnmirroredGrid gives the grid back exactly; the
    mirrored copy holds the cells mirrored, with the shifted link along the
    mirrored direction; the cone window resets the cells outside it; the
    Tukey window is 1 on its plateau and 0 outside."""
    from oracle import occupation as oc
    g = orc.OracleGrid(2, (4, 3, 5), dt=0.5)
    g.random_links(3, 0.3)
    g.random_e(3, 0.2)
    g.update_links()
    for md in range(3):
        m = oc.mirrored_grid(g, md)
        back = oc.unmirrored_grid(m, md, g.dims)
        for k in ("U", "Unext", "E"):
            assert np.array_equal(getattr(back, k), getattr(g, k))
        n = g.dims[md]
        x = np.indices(g.dims).reshape(3, -1)
        y = x.copy()
        y[md] = 2 * n - 1 - x[md]
        dm = m.dims
        i2 = (y[0] * dm[1] + y[1]) * dm[2] + y[2]
        assert np.array_equal(m.E[i2], g.E)
        z = x.copy()
        z[md] = np.maximum(z[md] - 1, 0)
        ish = (z[0] * g.dims[1] + z[1]) * g.dims[2] + z[2]
        assert np.array_equal(m.U[i2, md], g.U[ish, md])
    c = g.copy()
    oc.windows(c, oc.CONE, 1.0, 0.0, (1.0, 0.0, 0.0), (1.0, 0.0, 0.0), 0.0)
    x0 = np.arange(g.V) // (g.dims[1] * g.dims[2])
    outside = (x0 < 0) | (x0 > 2)
    assert np.all(c.U[outside] == np.array([1.0, 0, 0, 0])) and np.all(c.E[outside] == 0)
    assert np.array_equal(c.E[~outside], g.E[~outside])
    t = g.copy()
    # Tukey, width 0.5: plateau for |x| <= 0.25, zero for |x| >= 0.75 (x = (pos - c) / (maxPos - minPos))
    oc.windows(t, oc.TUKEY, 2.0, 0.0, (2.0, 0.0, 0.0), (1.0, 0.0, 0.0), 0.5)
    xx = (x0 * 1.0 - 2.0) / 4.0
    plateau = np.abs(xx) <= 0.25
    assert np.allclose(t.E[plateau], g.E[plateau], rtol=0, atol=0)


def _su3_from_herm(H):
    """exp(i H) for a 3x3 hermitian H, as 18 reals (re, im row-major)."""
    import scipy.linalg
    U = scipy.linalg.expm(1j * H)
    return np.concatenate([U.real.reshape(-1), U.imag.reshape(-1)])


def _gen_herm(x):
    """H = x_a lambda_a / 2 (Gell-Mann matrices)."""
    lam = np.zeros((8, 3, 3), complex)
    lam[0][0, 1] = lam[0][1, 0] = 1
    lam[1][0, 1], lam[1][1, 0] = -1j, 1j
    lam[2][0, 0], lam[2][1, 1] = 1, -1
    lam[3][0, 2] = lam[3][2, 0] = 1
    lam[4][0, 2], lam[4][2, 0] = -1j, 1j
    lam[5][1, 2] = lam[5][2, 1] = 1
    lam[6][1, 2], lam[6][2, 1] = -1j, 1j
    lam[7] = np.diag([1, 1, -2]) / np.sqrt(3)
    return np.einsum("a,aij->ij", x, lam) / 2


@pytest.mark.parametrize("scale", [1e-6, 0.05, 0.8, 2.5])
def test_su3_log_inverts_exp(orc, scale):
    """The oracle's SU(3) logarithm (SU3GroupElement.getAlgebraElement) returns
    the generator components x with exp(i x_a lambda_a / 2) = U: for random x
    of the given size (principal branch, |x| below pi) the components come back
    to 1e-12, near the identity too."""
    import ctypes as C
    from oracle import _p, lib
    L = lib()
    L.orc_su3_log_gen.argtypes = [C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(11)
    for _ in range(50):
        x = rng.normal(size=8)
        x *= scale / np.linalg.norm(x)
        u = _su3_from_herm(_gen_herm(x))
        g = np.empty(8)
        L.orc_su3_log_gen(_p(u), _p(g))
        assert np.abs(g - x).max() <= 1e-12 * max(1.0, scale), (x, g)


def test_su3_log_degenerate(orc):
    """Coincident eigenvalues: diag(e^{ia}, e^{ia}, e^{-2ia}) conjugated by a
    random unitary, and the identity."""
    import ctypes as C
    import scipy.stats
    from oracle import _p, lib
    L = lib()
    L.orc_su3_log_gen.argtypes = [C.c_void_p, C.c_void_p]
    W = scipy.stats.unitary_group.rvs(3, random_state=4)
    for a in (0.0, 0.3, 1.0):
        H = W @ np.diag([a, a, -2 * a]) @ W.conj().T
        u = _su3_from_herm(H)
        g = np.empty(8)
        L.orc_su3_log_gen(_p(u), _p(g))
        assert np.abs(_gen_herm(g) - H).max() <= 1e-12, a


def test_su3_log_phase_sum_2pi(orc):
    """Eigenphases whose principal values add up to 2 pi: the logarithm is
    still traceless and exp(i H) = U (one phase carries the 2 pi)."""
    import ctypes as C
    import scipy.linalg
    import scipy.stats
    from oracle import _p, lib
    L = lib()
    L.orc_su3_log_gen.argtypes = [C.c_void_p, C.c_void_p]
    W = scipy.stats.unitary_group.rvs(3, random_state=7)
    H0 = W @ np.diag([2.3, 2.2, -4.5]) @ W.conj().T
    u = _su3_from_herm(H0)
    g = np.empty(8)
    L.orc_su3_log_gen(_p(u), _p(g))
    H = _gen_herm(g)
    assert abs(np.trace(H)) < 1e-12
    U1 = scipy.linalg.expm(1j * H)
    U0 = (u[:9] + 1j * u[9:]).reshape(3, 3)
    assert np.abs(U1 - U0).max() < 1e-12


def test_su3_coulomb_gauge_removes_pure_gauge(orc):
    """SU(3): links U_i(x) = g(x) g(x+i)^dagger of a random gauge function g and
    E = 0 are pure gauge; the Coulomb gauge iteration drives the divergence
    below the goal and the occupation numbers and energy to zero."""
    import ctypes as C
    from oracle import _p, lib, occupation
    g = orc.OracleGrid(3, (4, 5, 6), dt=0.1)
    rng = np.random.default_rng(2)
    V = g.V
    G = np.empty((V, 18))
    L = lib()
    for x in range(V):
        G[x] = _su3_from_herm(_gen_herm(rng.normal(0, 0.15, 8)))
    def cm(v):
        return (v[:9] + 1j * v[9:]).reshape(3, 3)
    for x in range(V):
        for d in range(3):
            xs = g.shift(x, d, 1)
            M = cm(G[x]) @ cm(G[xs]).conj().T
            g.U[x, d] = np.concatenate([M.real.reshape(-1), M.imag.reshape(-1)])
    g.Unext[...] = g.U
    n, e, conv = occupation.occupation_numbers(g, max_iter=200, goal=1e-20)
    assert conv[-1] < 1e-20
    assert np.abs(n).max() < 1e-12 and abs(e) < 1e-12
