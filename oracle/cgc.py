"""CPU oracle of the CGC (MV-model) initial condition.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` and the benchmark's CPU legs;
the GPU product never imports it.

Restates, for one MV nucleus at a time (paths relative to
pixi/src/main/java/org/openpixi/pixi):

* physics/initial/CGC/MVModel.java:101-157 -- random charges (``orc_mv_charges``,
  java.util.Random restated in C), 3D momentum-space regulation, longitudinal
  window;
* physics/initial/CGC/FourierFunctions.java:86-172 -- ``regulate`` and
  ``poisson2d`` below, with numpy's FFT in place of JTransforms 2.4.0
  (com.github.rwl:jtransforms, the reference's FFT dependency, absent here):
  a complex forward transform, a real even multiplier, and a scaled complex
  inverse transform, whose real part is kept;
* physics/initial/CGC/LightConePoissonSolverImproved.java:42-221 -- per-sheet
  Poisson solves here, the rest in ``orc_cgc_solve``;
* physics/initial/CGC/LightConeNGPParticleCreator.java:110-305 --
  ``orc_cgc_particles``;
* physics/initial/CGC/CGCInitialCondition.java:55-93 -- the order of the three.
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import OracleGrid, OracleParticles, _p, lib, na, ng, ngen


@dataclass
class MVNucleus:
    """MVModel constructor arguments (MVModel.java:84-99)."""
    orientation: int
    location: float
    width: float
    mu: float
    seed: int
    uvt: float = 4.44
    coherence: float = 0.0
    ir: float = 0.0
    direction: int = 0


def java_random(seed, kind, count):
    """java.util.Random(seed): kind 0 nextGaussian, 1 nextDouble, 2 nextInt."""
    out = np.empty(count)
    L = lib()
    L.orc_java_random.argtypes = [C.c_int64, C.c_int, C.c_long, C.c_void_p]
    L.orc_java_random(seed, kind, count, _p(out))
    return out


def _kt(n1, n2, aT):
    """computeEffectiveTransverseMomentumSquared and computeTransverseMomentumSquared
    (FourierFunctions.java:182-219) on the transverse grid."""
    t1 = np.arange(n1)[:, None]
    t2 = np.arange(n2)[None, :]
    kTeff2 = 2.0 * 2
    kTeff2 = kTeff2 - 2.0 * np.cos((2.0 * np.pi * t1) / n1)
    kTeff2 = kTeff2 - 2.0 * np.cos((2.0 * np.pi * t2) / n2)
    kTeff2 = kTeff2 / (aT * aT)
    twopi = 2.0 * np.pi
    k1 = np.where(t1 < n1 // 2, twopi * t1 / (aT * n1), twopi * (n1 - t1) / (aT * n1))
    k2 = np.where(t2 < n2 // 2, twopi * t2 / (aT * n2), twopi * (n2 - t2) / (aT * n2))
    kT2 = k1 * k1 + k2 * k2
    return np.broadcast_to(kTeff2, (n1, n2)), kT2


def regulate(rho, dims, uvt, long_width, ir, aT, aL):
    """FourierFunctions.regulateChargeDensityGaussian (:86-132), beam along dimension 0."""
    n0, n1, n2 = dims
    f = np.fft.fftn(rho.reshape(dims).astype(complex))
    kTeff2, kT2 = _kt(n1, n2, aT)
    delta = np.arange(n0) / float(n0)
    kL = np.abs(np.where(delta < 0.5, 2.0 * delta * np.pi / aL, 2.0 * (delta - 1.0) * np.pi / aL))
    with np.errstate(invalid="ignore", divide="ignore"):
        reg = (kTeff2 / (kTeff2 + ir * ir))[None, :, :] * np.exp(-0.25 * kL * kL * long_width * long_width)[:, None, None]
    keep = ((kT2 <= uvt * uvt) & (kT2 > 0))[None, :, :]
    f = np.where(keep, f * reg, 0.0)
    f[0, 0, 0] = 0.0
    return np.fft.ifftn(f).real.reshape(-1)


def poisson2d(rho, dims, aT):
    """FourierFunctions.solvePoisson2D (:147-172) on every longitudinal sheet."""
    n0, n1, n2 = dims
    f = np.fft.fft2(rho.reshape(dims).astype(complex), axes=(1, 2))
    kTeff2, _ = _kt(n1, n2, aT)
    inv = np.zeros((n1, n2))
    inv.flat[1:] = 1.0 / kTeff2.flat[1:]
    f = f * inv[None]
    return np.fft.ifft2(f, axes=(1, 2)).real.reshape(-1)


def mv_nucleus(grid: OracleGrid, nu: MVNucleus, super_particles=False):
    """CGCInitialCondition.applyInitialCondition for one MVModel: updates the
    grid's U, Unext, E and returns the new particles (OracleParticles), or the
    nucleus's super-particle group (SuperGroup) for the optimized simulation type."""
    if nu.direction != 0:
        raise ValueError("the particle creator assumes the beam along dimension 0")
    L = lib()
    V, nc, dims = grid.V, grid.nc, grid.dims
    k = ngen(nc)
    aL, aT = grid.a[0], grid.a[1]
    raw = np.empty((k, V))
    L.orc_mv_charges.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int64, C.c_void_p]
    L.orc_mv_charges(grid.pp, 0, nu.location, nu.width, nu.mu, int(nu.seed), _p(raw))
    # regulation and the window lmin < z < lmax on active cells (MVModel.java:134-153)
    box = dims[0] * aL
    zmin = max(nu.location - box / 2.0, 0.0)
    zmax = min(nu.location + box / 2.0, box)
    lmin, lmax = int(np.floor(zmin / aL)), int(np.ceil(zmax / aL))
    z = np.arange(V) // (dims[1] * dims[2])
    keep = (lmin < z) & (z < lmax) & (grid.active != 0)
    rho = np.zeros((k, V))
    for c in range(k):
        r = regulate(raw[c], dims, nu.uvt, nu.coherence, nu.ir, aT, aL)
        rho[c] = np.where(keep, r, 0.0)
    phi = np.ascontiguousarray(np.stack([poisson2d(rho[c], dims, aT) for c in range(k)]))
    gauss = np.empty((V, na(nc)))
    vt = np.empty((dims[1] * dims[2], ng(nc)))
    L.orc_cgc_solve.argtypes = [C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 7
    L.orc_cgc_solve(grid.pp, 0, int(nu.orientation), _p(phi), _p(grid.U), _p(grid.Unext), _p(grid.E),
                    _p(grid.active), _p(gauss), _p(vt))
    info = {"rho": rho, "phi": phi, "gauss": gauss, "vt": vt}
    if super_particles:
        return super_group(grid, gauss, int(nu.orientation)), info
    L.orc_cgc_particles.restype = C.c_long
    L.orc_cgc_particles.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_long] + [C.c_void_p] * 4
    n = L.orc_cgc_particles(grid.pp, _p(gauss), int(nu.orientation), 0, None, None, None, None)
    if n < 0:
        raise ValueError("round(aL/dt) particles per cell must be >= 1")
    P = OracleParticles(nc, n)
    L.orc_cgc_particles(grid.pp, _p(gauss), int(nu.orientation), n, _p(P.pos0), _p(P.pos1), _p(P.vel), _p(P.Q0))
    P.Q1[...] = P.Q0
    P.dir[...] = 0
    return P, info


def wilson_tadpole(vt, nc):
    """WilsonLineObservables.computeTadpole (physics/initial/CGC/WilsonLineObservables.java:37-59)."""
    L = lib()
    L.orc_wilson_tadpole.restype = C.c_double
    L.orc_wilson_tadpole.argtypes = [C.c_int, C.c_void_p, C.c_long]
    v = np.ascontiguousarray(vt, dtype=np.float64)
    return L.orc_wilson_tadpole(nc, _p(v), v.shape[0])


def wilson_dipole(vt, nc, n1, n2, a1=1.0, a2=1.0):
    """WilsonLineObservables.computeDipole (:67-131): (bin values, bin width)."""
    L = lib()
    L.orc_wilson_dipole.restype = C.c_int
    L.orc_wilson_dipole.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double,
                                    C.c_void_p, C.c_void_p]
    v = np.ascontiguousarray(vt, dtype=np.float64)
    nb = L.orc_wilson_dipole(nc, _p(v), n1, n2, a1, a2, None, None)
    out = np.empty(max(nb, 1))
    ds = C.c_double()
    L.orc_wilson_dipole(nc, _p(v), n1, n2, a1, a2, _p(out), C.byref(ds))
    return out[:nb], ds.value


class SuperGroup:
    """The super particles of one nucleus (LightConeNGPSuperParticleCreator):
    Q[k][i] is charge i of super particle k, i over the particle block
    [base, base + n) of global cell indices."""

    def __init__(self, orientation, n, base, Q):
        self.orientation = orientation
        self.n = n
        self.base = base
        self.Q = Q


def super_group(grid, gauss, orientation):
    L = lib()
    L.orc_super_create.restype = C.c_long
    L.orc_super_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    base = C.c_long()
    n = L.orc_super_create(grid.pp, _p(gauss), C.byref(base), None)
    if n < 0:
        raise ValueError("round(aL/dt) particles per cell must be >= 1")
    ppc = int(round(grid.a[0] / grid.dt))
    Q = np.zeros((ppc, max(n, 1), na(grid.nc)))
    L.orc_super_create(grid.pp, _p(gauss), C.byref(base), _p(Q))
    return SuperGroup(orientation, n, base.value, Q)


class OracleSuperSimulation:
    """Simulation.initialize/step (physics/Simulation.java:318-435) for the
    optimized CGC type: field update, then CGCSuperParticleInterpolationNGP's
    charge density and current (the particle solver does nothing)."""

    def __init__(self, grid, groups, nthreads=1, implicit=None):
        self.grid = grid
        self.groups = groups
        self.nthreads = nthreads
        self.steps = 0
        self.implicit = implicit  # (iterations, damping) for ImplicitTYMSolver

    def _args(self):
        k = len(self.groups)
        orient = (C.c_int * k)(*[g.orientation for g in self.groups])
        n = (C.c_long * k)(*[g.n for g in self.groups])
        base = (C.c_long * k)(*[g.base for g in self.groups])
        Q = (C.c_void_p * k)(*[g.Q.ctypes.data for g in self.groups])
        return k, orient, n, base, Q

    def _phases(self, t):
        g, L = self.grid, lib()
        k, orient, n, base, Q = self._args()
        L.orc_super_cin.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int, C.c_long, C.c_void_p]
        L.orc_super_jin.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int, C.c_long, C.c_void_p, C.c_void_p]
        g.rho[...] = 0.0
        L.orc_super_cin(g.pp, k, orient, n, base, Q, self.nthreads, t, _p(g.rho))
        g.J[...] = 0.0
        L.orc_super_jin(g.pp, k, orient, n, base, Q, self.nthreads, t, _p(g.Unext), _p(g.J))

    def initialize(self):
        self.grid.update_links()
        self._phases(0)

    def step(self):
        self.steps += 1
        self.grid.store_fields()
        if self.implicit is not None:
            self.grid.update_grid_implicit(*self.implicit)
        else:
            self.grid.update_grid()
        self._phases(self.steps)


def cgc_mv_super(grid: OracleGrid, nuclei):
    """All nuclei in order, with super particles (simulationType temporal optimized cgc ngp)."""
    groups, info = [], []
    for nu in nuclei:
        G, d = mv_nucleus(grid, nu, super_particles=True)
        groups.append(G)
        info.append(d)
    return groups, info


def concat(parts, nc):
    n = sum(p.n for p in parts)
    out = OracleParticles(nc, n)
    o = 0
    for p in parts:
        for key in ("pos0", "pos1", "vel", "Q0", "Q1", "dir"):
            getattr(out, key)[o:o + p.n] = getattr(p, key)
        o += p.n
    return out


def cgc_mv(grid: OracleGrid, nuclei):
    """All nuclei in order (one CGCInitialCondition per YAML MVModel entry)."""
    parts, info = [], []
    for nu in nuclei:
        P, d = mv_nucleus(grid, nu)
        parts.append(P)
        info.append(d)
    return concat(parts, grid.nc), info
