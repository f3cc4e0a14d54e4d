"""Pins the CPU oracle to the reference's own tests (restated) and to an
independent matrix library (numpy/scipy standing in for the commons-math3
matrices of the reference's math tests).

Reference tests restated here (paths relative to pixi/src/test/java/org/openpixi/pixi):
  math/SU2MatrixTest.java (accuracy 1e-13), math/SU2FieldTest.java (1e-14),
  math/SU3EverythingTest.java (1e-12; exp against a 100-term series :238-277),
  physics/grid/GridTest.java (1e-13: link/plaquette identities, index maps, shift),
  physics/grid/GaussConstraintTest.java (analytic |div E|^2 under random gauge
  transformations, 1e-4).
"""
import numpy as np
import pytest
import scipy.linalg as sla

SIG = [np.array([[0, 1], [1, 0]], complex), np.array([[0, -1j], [1j, 0]]), np.array([[1, 0], [0, -1]], complex)]
LAM = [np.array(m, complex) for m in (
    [[0, 1, 0], [1, 0, 0], [0, 0, 0]], [[0, -1j, 0], [1j, 0, 0], [0, 0, 0]],
    [[1, 0, 0], [0, -1, 0], [0, 0, 0]], [[0, 0, 1], [0, 0, 0], [1, 0, 0]],
    [[0, 0, -1j], [0, 0, 0], [1j, 0, 0]], [[0, 0, 0], [0, 0, 1], [0, 1, 0]],
    [[0, 0, 0], [0, 0, -1j], [0, 1j, 0]])] + [np.diag([1, 1, -2]).astype(complex) / np.sqrt(3)]


def su2_mat(q):
    return q[0] * np.eye(2) + 1j * sum(q[k + 1] * SIG[k] for k in range(3))


def su3_mat(e):
    return (np.array(e[:9]) + 1j * np.array(e[9:])).reshape(3, 3)


def mat(nc, u):
    return su2_mat(u) if nc == 2 else su3_mat(u)


def alg_mat(nc, orc, v):
    """Hermitian matrix X = x^a t_a of an algebra element in the reference layout."""
    g = orc.alg_to_gen(nc, v)
    T = SIG if nc == 2 else LAM
    return sum(g[a] * T[a] / 2 for a in range(len(g)))


def rand_group(nc, rng, scale=1.0):
    T = SIG if nc == 2 else LAM
    H = sum(rng.normal(0, scale) * t / 2 for t in T)
    M = sla.expm(1j * H)
    if nc == 2:
        return np.array([M[0, 0].real, M[0, 1].imag, M[0, 1].real, M[0, 0].imag]), M
    return np.concatenate([M.real.ravel(), M.imag.ravel()]), M


@pytest.mark.parametrize("nc", [2, 3])
def test_group_ops_match_matrices(orc, nc):
    rng = np.random.default_rng(11 + nc)
    tol = 1e-13 if nc == 2 else 1e-12
    for _ in range(50):
        a, A = rand_group(nc, rng)
        b, B = rand_group(nc, rng)
        assert np.allclose(mat(nc, a), A, atol=1e-14)
        assert np.abs(mat(nc, orc.group_mult(nc, a, b)) - A @ B).max() < tol
        assert np.abs(mat(nc, orc.group_adj(nc, a)) - A.conj().T).max() < tol
        # unitarity (SU2MatrixTest :63)
        assert np.abs(A @ A.conj().T - np.eye(nc)).max() < tol
        # proj: proj_a(M) = Im tr(lambda_a M) (generator components)
        T = SIG if nc == 2 else LAM
        pg = orc.alg_to_gen(nc, orc.group_proj(nc, a))
        assert np.allclose(pg, [np.trace(t @ A).imag for t in T], atol=tol)


@pytest.mark.parametrize("nc", [2, 3])
@pytest.mark.parametrize("scale", [0.05, 0.6, 2.5])
def test_getlink_is_exp(orc, nc, scale):
    """getLink(X) = exp(i X^a t_a); SU(3) covers both the Taylor (tr X^2 <= 1) and the
    eigen-decomposition branch (SU3EverythingTest.testAlgebraGroupElements :238-277)."""
    rng = np.random.default_rng(5)
    for _ in range(30):
        g = rng.normal(0, scale, 3 if nc == 2 else 8)
        v = orc.gen_to_alg(nc, g)
        U = mat(nc, orc.alg_getlink(nc, v))
        X = alg_mat(nc, orc, v)
        assert np.abs(U - sla.expm(1j * X)).max() < (1e-13 if nc == 2 else 1e-11)


@pytest.mark.parametrize("nc", [2, 3])
def test_act_is_conjugation(orc, nc):
    """act(X, g) = g X g^dagger (SU2MatrixTest :363, SU3EverythingTest :356)."""
    rng = np.random.default_rng(7)
    for _ in range(30):
        a, A = rand_group(nc, rng)
        v = orc.gen_to_alg(nc, rng.normal(0, 1, 3 if nc == 2 else 8))
        X = alg_mat(nc, orc, v)
        Y = alg_mat(nc, orc, orc.alg_act(nc, v, a))
        assert np.abs(Y - A @ X @ A.conj().T).max() < 1e-12


def test_su3_generator_roundtrip(orc):
    rng = np.random.default_rng(3)
    for _ in range(20):
        g = rng.normal(0, 1, 8)
        assert np.allclose(orc.alg_to_gen(3, orc.gen_to_alg(3, g)), g, atol=1e-15)
        # square() = sum of squared generator components (SU3AlgebraElement.square :174-176)
        assert abs(orc.alg_square(3, orc.gen_to_alg(3, g)) - (g ** 2).sum()) < 1e-13


def _grid(orc, nc, dims, seed=1, sigma=0.3, dt=0.05):
    g = orc.OracleGrid(nc, dims, dt=dt)
    g.random_links(seed, sigma)
    g.random_e(seed, sigma)
    return g


def test_grid_index_and_shift(orc):
    """GridTest.testCellIndexMethods / testShiftAndPeriodic on the 16x17x18 lattice."""
    g = orc.OracleGrid(2, (16, 17, 18))
    n = np.array(g.dims)
    rng = np.random.default_rng(0)
    for _ in range(200):
        pos = rng.integers(0, n)
        idx = (pos[0] * n[1] + pos[1]) * n[2] + pos[2]
        for d in range(3):
            for o in (1, -1):
                p2 = pos.copy()
                p2[d] = (p2[d] + o) % n[d]
                assert g.shift(idx, d, o) == (p2[0] * n[1] + p2[1]) * n[2] + p2[2]


def test_grid_link_and_plaquette_identities(orc):
    """GridTest.testLinkMethods: getLink forward/backward consistency, P_ij P_ji = 1,
    and forward/backward plaquettes around one rectangle have the same trace."""
    g = _grid(orc, 2, (16, 17, 18), seed=4, sigma=1.0)
    rng = np.random.default_rng(1)
    for _ in range(50):
        idx = int(rng.integers(0, g.V))
        d1, d2 = (int(x) for x in rng.integers(0, 3, 2))
        p1 = g.plaquette(idx, d1, d2, 1, 1)
        p2 = g.plaquette(idx, d2, d1, 1, 1)
        r = orc.group_mult(2, p1, p2)
        assert np.allclose(r, [1, 0, 0, 0], atol=1e-13)
        p3 = g.plaquette(g.shift(idx, d1, 1), d1, d2, -1, 1)
        assert abs(p1[0] - p3[0]) < 1e-13


def _gauge_transform(orc, g, seed):
    """Random gauge transformation U_i(x) -> h(x) U_i(x) h(x+i)^dagger, E -> h E h^dagger
    (the test tool gauge/RandomGauge.java + GaugeTransformation.java)."""
    nc = g.nc
    rng = np.random.default_rng(seed)
    hs = [rand_group(nc, rng, 1.0)[0] for _ in range(g.V)]
    U = g.U.copy()
    for x in range(g.V):
        for i in range(3):
            y = g.shift(x, i, 1)
            g.U[x, i] = orc.group_mult(nc, orc.group_mult(nc, hs[x], U[x, i]), orc.group_adj(nc, hs[y]))
            g.E[x, i] = orc.alg_act(nc, g.E[x, i], hs[x])


def test_gauss_constraint_analytic(orc):
    """GaussConstraintTest.testGaussConstraintViolation: E_i^a(x) = A_i B^a n.x on a
    16x16x1 lattice (a = 0.05, dt = 0.00025, g = 1).  |div E|^2 = |B|^2 (A.n)^2 in the
    interior, invariant under random gauge transformations and under the evolution."""
    a, dt = 0.05, 0.00025
    g = orc.OracleGrid(2, (16, 16, 1), a=a, dt=dt)
    A = np.array([0.345345, 0.0, 0.0])
    B = np.array([0.2345245, 0.02343, -1.234])
    n = np.array([1.567, 0.534, 0.0])
    for x in range(g.V):
        pos = np.array([x // 16, x % 16, 0])
        nx = (pos * a * n).sum()
        for j in range(3):
            g.E[x, j] = A[j] * B * 1.0 * a * nx
    g.update_links()
    expected = (B ** 2).sum() * (A @ n) ** 2
    sim = orc.OracleSimulation(g)
    for step in range(40):
        if step % 10 == 0:
            _gauge_transform(orc, g, step)
            g.update_links()
        for _ in range(5):
            px, py = np.random.default_rng(step).integers(4, 12, 2)
            val = orc.alg_square(2, g.gauss_constraint(int(px * 16 + py)))
            assert abs(val - expected) < 1e-4
        sim.step()


@pytest.mark.parametrize("nc", [2, 3])
def test_gauss_projection_and_conservation(orc, nc):
    g = _grid(orc, nc, (6, 6, 6), seed=9, sigma=0.3)
    assert g.bulk()[9] > 1e-3
    it, g2 = g.gauss_project(tol_g2=1e-26)
    assert g2 < 1e-26 and it < 1000
    sim = orc.OracleSimulation(g)
    sim.initialize()
    for _ in range(20):
        sim.step()
    assert g.bulk()[9] < 1e-24


def test_restoration_reduces_violation(orc):
    """GaussConstraintRestoration.iterateRestorationAlgorithm lowers the violation
    monotonically (rolls back otherwise)."""
    g = _grid(orc, 2, (6, 6, 6), seed=2, sigma=0.2)
    g.update_links()
    from oracle import lib
    import ctypes as C
    gv = np.empty((g.V, 4))
    it, v = g.gauss_restoration(gamma=0.2, maxit=200, absval=1e-20)
    g2 = g.copy()
    it2, v2 = g2.gauss_restoration(gamma=0.2, maxit=1, absval=1e-20)
    assert it > 10 and v < 1e-3 * 0.5


@pytest.mark.parametrize("nc", [2, 3])
def test_hamiltonian_conserved(orc, nc):
    """The leapfrog conserves H = sum E^2/2 + 2 sum_plaq (N - Re tr P) up to O(dt^2)
    oscillation: a check of the restated update equations independent of the reference."""
    g = _grid(orc, nc, (4, 4, 4), seed=3, sigma=0.3, dt=0.02)
    g.gauss_project()
    sim = orc.OracleSimulation(g)
    sim.initialize()

    def H():
        e2 = (g.e_gen() ** 2).sum() / 2
        v = 0.0
        for x in range(g.V):
            for i in range(3):
                for j in range(i + 1, 3):
                    for t in (0, 1):
                        P = g.plaquette(x, i, j, 1, 1, t)
                        tr = 2 * P[0] if nc == 2 else P[0] + P[4] + P[8]
                        v += 0.5 * (nc - tr)
        return e2 + 2 * v

    h0 = H()
    hs = []
    for _ in range(30):
        sim.step()
        hs.append(H())
    assert np.max(np.abs(np.array(hs) - h0)) / h0 < 2e-3


def test_ngp_rounds_half_even(orc):
    g = orc.OracleGrid(2, (8, 8, 8))
    P = orc.OracleParticles(2, 1)
    pos = np.array([[0.5, 1.5, 2.5], [2.4999, -0.5, 7.5000001]])
    c = P.ngp(g, pos)
    assert c.tolist() == [[0, 2, 2], [2, 0, 8]]


# ---------------------------------------------------------------- Poynting rows
def _su2_mat(q):
    """quaternion (e0, e1, e2, e3) -> e0 + i e.sigma as a 2x2 complex matrix"""
    e0, e1, e2, e3 = q
    return np.array([[e0 + 1j * e3, e2 + 1j * e1], [-e2 + 1j * e1, e0 - 1j * e3]])


def _su2_proj(M):
    """2 (e1, e2, e3) of a real-linear combination of SU(2) matrices"""
    return 2.0 * np.array([M[0, 1].imag, M[0, 1].real, M[0, 0].imag])


_SIG = [np.array([[0, 1], [1, 0]], complex), np.array([[0, -1j], [1j, 0]]), np.array([[1, 0], [0, -1]], complex)]


def _alg_mat(v):
    return sum(v[a] * _SIG[a] for a in range(3)) / 2.0


def _alg_vec(X):
    return np.array([np.trace(_SIG[a] @ X).real for a in range(3)])


def test_poynting_rows_against_independent_matrices(orc):
    """ProjectedEnergyDensity.PoyntingComputation (ProjectedEnergyDensity.java:182-279)
    restated a second time with numpy 2x2 matrices on a small uneven SU(2) lattice."""
    dims, a, g_, dt = (4, 3, 5), (1.0, 0.9, 1.2), 1.3, 0.1
    g = orc.OracleGrid(2, dims, a=a, dt=dt, g=g_)
    g.random_links(3, 0.7)
    g.random_e(3, 0.5)
    g.update_links()
    # the independent 2x2 form must agree with the oracle's act first
    X = _alg_mat(g.E[7, 1])
    Um = _su2_mat(g.U[5, 2])
    assert np.allclose(_alg_vec(Um @ X @ Um.conj().T), orc.alg_act(2, g.E[7, 1], g.U[5, 2]), atol=1e-13)
    V = g.V

    def idx(p):
        return ((p[0] % dims[0]) * dims[1] + (p[1] % dims[1])) * dims[2] + (p[2] % dims[2])

    def link(W, p, d, o):
        if o > 0:
            return _su2_mat(W[idx(p), d])
        q = list(p); q[d] -= 1
        return _su2_mat(W[idx(q), d]).conj().T

    def plaq(W, p, d1, d2, o1, o2):
        x1 = list(p)
        x2 = list(x1); x2[d1] += o1
        x3 = list(x2); x3[d2] += o2
        x4 = list(x3); x4[d1] -= o1
        return link(W, x1, d1, o1) @ link(W, x2, d2, o2) @ link(W, x3, d1, -o1) @ link(W, x4, d2, -o2)

    for d in range(3):
        N = dims[d]
        area = V / N
        ufF = [1.0 / ((a[i] * a[d]) * g_ * np.sqrt(area)) for i in range(3)]
        ufEB = [1.0 / ((g_ * a[i]) * np.sqrt(area)) for i in range(3)]
        avg, tavg = np.zeros(N), np.zeros(N)
        for x in range(V):
            p = [x // (dims[1] * dims[2]), (x // dims[2]) % dims[1], x % dims[2]]
            la = 0.0
            for i in range(3):
                if i == d:
                    continue
                FG = np.zeros((2, 2), complex)
                for W in (g.U, g.Unext):
                    FG += plaq(W, p, d, i, 1, 1) + plaq(W, p, i, d, -1, 1) + plaq(W, p, i, d, 1, -1) \
                        + plaq(W, p, d, i, -1, -1)
                F = _su2_proj(FG) * ufF[i] / 8.0
                q = list(p); q[i] -= 1
                Ub = link(g.U, p, i, -1)
                E2 = _alg_vec(Ub @ _alg_mat(g.E[idx(q), i]) @ Ub.conj().T)
                la += np.dot((g.E[x, i] + E2) * 0.5 * ufEB[i], F)
            d1, d2 = (d + 1) % 3, (d + 2) % 3

            def bvec(W, dd):
                j, k = (dd + 1) % 3, (dd + 2) % 3
                return _su2_proj(plaq(W, p, j, k, 1, 1)) * a[dd] / (a[j] * a[k])
            B1 = (bvec(g.U, d1) + bvec(g.Unext, d1)) * ufEB[d1] * 0.5
            B2 = (bvec(g.U, d2) + bvec(g.Unext, d2)) * ufEB[d2] * 0.5
            ta = np.dot(g.E[x, d1] * ufEB[d1], B2) - np.dot(g.E[x, d2] * ufEB[d2], B1)
            avg[p[d]] += la
            tavg[p[d]] += ta
        ref = np.stack([avg, tavg])
        got = g.projected_poynting(d)
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max()), (d, got, ref)
        assert np.abs(ref).max() > 1e-4


@pytest.mark.parametrize("nc", [2, 3])
def test_implicit_solver_properties(orc, nc):
    """ImplicitTYMSolver (physics/fields/ImplicitTYMSolver.java): with no
    iterations it is the explicit FastTYMSolver update bit for bit (ImplicitBegin
    is the CombinedUpdate); with iterations and no damping the fixed-point
    iteration converges (successive iterates approach each other)."""
    g = orc.OracleGrid(nc, (6, 6, 6) if nc == 2 else (4, 4, 5), dt=0.05)
    g.random_links(3, 0.3)
    g.random_e(3, 0.3)
    g.gauss_project()
    a, b = g.copy(), g.copy()
    sa = orc.OracleSimulation(a)
    sb = orc.OracleSimulation(b, implicit=(0, 0.0))
    sa.initialize()
    sb.initialize()
    for _ in range(4):
        sa.step()
        sb.step()
    assert np.array_equal(a.U.view(np.uint64), b.U.view(np.uint64))
    assert np.array_equal(a.E.view(np.uint64), b.E.view(np.uint64))
    diffs = []
    for it in (4, 8, 12):
        c = g.copy()
        sc = orc.OracleSimulation(c, implicit=(it, 0.0))
        sc.initialize()
        sc.step()
        diffs.append(c.Unext.copy())
    assert np.abs(diffs[2] - diffs[1]).max() < np.abs(diffs[1] - diffs[0]).max()


@pytest.mark.parametrize("nc", [2, 3])
def test_temporal_ym_solver_equals_fast_solver(orc, nc):
    """TemporalYangMillsSolver (plaquette form, TemporalYangMillsSolver.java:49-95)
    and FastTYMSolver (staple form, FastTYMSolver.java:40-84) are the same
    update: after 6 steps on an uneven lattice with a current and an activity
    mask, links and E agree to FP64 rounding (1e-13)."""
    import numpy as np
    from helpers import oracle_ic, fresh, link_rel_err, field_rel_err
    g = fresh(oracle_ic(nc, (5, 4, 6), 13, 0.3, 0.3, a=(1.0, 1.2, 0.8)))
    rng = np.random.default_rng(3)
    g.J[...] = rng.normal(0, 0.05, g.J.shape)
    g.active[:] = (np.arange(g.V) % 7 != 4).astype(np.uint8)
    t = g.copy()
    g.update_links()
    t.update_links()
    for _ in range(6):
        g.store_fields()
        g.update_grid()
        t.store_fields()
        t.update_grid_tym()
    assert link_rel_err(t.Unext, g.Unext) <= 1e-13
    assert field_rel_err(t.E, g.E) <= 1e-13
