"""ctypes binding of the CPU FP64 oracle.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``.  The GPU product never imports it.

The classes mirror the reference's objects in its own (per-cell) layout:
``OracleGrid`` follows physics/grid/Grid.java + physics/fields/FastTYMSolver.java,
``OracleParticles`` the CGC particle list, and ``OracleSimulation`` the phase
order of physics/Simulation.java:318-435.
"""
import ctypes as C
import os

import numpy as np

from .build_oracle import build as _build, LIB as _LIB

_lib = None


class _Params(C.Structure):
    _fields_ = [("nc", C.c_int), ("n", C.c_int * 3), ("a", C.c_double * 3),
                ("dt", C.c_double), ("g", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        _build()
        _lib = C.CDLL(_LIB)
        dp = C.POINTER(C.c_double)
        L = _lib
        L.orc_shift.restype = C.c_long
        L.orc_shift.argtypes = [C.POINTER(_Params), C.c_long, C.c_int, C.c_int]
        L.orc_alg_square.restype = C.c_double
        L.orc_normal.restype = C.c_double
        L.orc_normal.argtypes = [C.c_uint64, C.c_uint64]
        L.orc_random_gen.argtypes = [C.c_uint64, C.c_uint64, C.c_long, C.c_double, dp]
        L.orc_gauss_project_cg.restype = C.c_int
        L.orc_gauss_project_cg.argtypes = [C.POINTER(_Params), dp, dp, dp, C.c_double, C.c_int, dp]
        L.orc_gauss_restoration.restype = C.c_int
        L.orc_gauss_restoration.argtypes = [C.POINTER(_Params), dp, dp, dp, dp, C.c_double,
                                            C.c_int, C.c_double, dp]
        L.orc_max_threads.restype = C.c_int
    return _lib


def _p(a):
    """Pointer to a C-contiguous numpy array (None passes NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def ng(nc):
    return 18 if nc == 3 else 4


def na(nc):
    return 9 if nc == 3 else 3


def ngen(nc):
    return 8 if nc == 3 else 3


# ---------------------------------------------------------------- group math
def group_mult(nc, l, r):
    out = np.empty(ng(nc))
    lib().orc_group_mult(nc, _p(np.ascontiguousarray(l, float)), _p(np.ascontiguousarray(r, float)), _p(out))
    return out


def group_adj(nc, u):
    out = np.empty(ng(nc))
    lib().orc_group_adj(nc, _p(np.ascontiguousarray(u, float)), _p(out))
    return out


def group_proj(nc, u):
    out = np.empty(na(nc))
    lib().orc_group_proj(nc, _p(np.ascontiguousarray(u, float)), _p(out))
    return out


def alg_getlink(nc, v):
    out = np.empty(ng(nc))
    lib().orc_alg_getlink(nc, _p(np.ascontiguousarray(v, float)), _p(out))
    return out


def alg_act(nc, v, g):
    out = np.empty(na(nc))
    lib().orc_alg_act(nc, _p(np.ascontiguousarray(v, float)), _p(np.ascontiguousarray(g, float)), _p(out))
    return out


def alg_square(nc, v):
    lib().orc_alg_square.argtypes = [C.c_int, C.c_void_p]
    return lib().orc_alg_square(nc, _p(np.ascontiguousarray(v, float)))


def alg_to_gen(nc, v):
    out = np.empty(ngen(nc))
    lib().orc_alg_to_gen(nc, _p(np.ascontiguousarray(v, float)), _p(out))
    return out


def gen_to_alg(nc, gvec):
    out = np.empty(na(nc))
    lib().orc_gen_to_alg(nc, _p(np.ascontiguousarray(gvec, float)), _p(out))
    return out


def random_gen(seed, stream, count, sigma):
    out = np.empty(count)
    lib().orc_random_gen(C.c_uint64(seed), C.c_uint64(stream), count, sigma,
                         out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


# ---------------------------------------------------------------- lattice
class OracleGrid:
    """Lattice state in the reference layout (see opx_oracle.h)."""

    def __init__(self, nc, dims, a=1.0, dt=0.05, g=1.0):
        self.nc = nc
        self.dims = tuple(int(d) for d in dims)
        self.a = tuple(float(x) for x in (a if np.ndim(a) else (a, a, a)))
        self.dt = float(dt)
        self.g = float(g)
        self.V = int(np.prod(self.dims))
        self.params = _Params(nc, (C.c_int * 3)(*self.dims), (C.c_double * 3)(*self.a), self.dt, self.g)
        V, G, A = self.V, ng(nc), na(nc)
        ident = np.zeros(G)
        ident[[0, 4, 8] if nc == 3 else [0]] = 1.0
        self.U = np.tile(ident, (V, 3, 1)).copy()
        self.Unext = self.U.copy()
        self.E = np.zeros((V, 3, A))
        self.J = np.zeros((V, 3, A))
        self.rho = np.zeros((V, A))
        self.active = np.ones(V, np.uint8)
        self.eval = np.ones(V, np.uint8)

    @property
    def pp(self):
        return C.byref(self.params)

    def copy(self):
        o = OracleGrid(self.nc, self.dims, self.a, self.dt, self.g)
        for k in ("U", "Unext", "E", "J", "rho", "active", "eval"):
            setattr(o, k, getattr(self, k).copy())
        return o

    # physics/grid/Grid.java
    def shift(self, index, d, o):
        return lib().orc_shift(self.pp, index, d, o)

    def staple_sum(self, index, d):
        out = np.empty(ng(self.nc))
        lib().orc_staple_sum(self.pp, _p(self.U), C.c_long(index), d, _p(out))
        return out

    def plaquette(self, index, d1, d2, o1, o2, t=0):
        out = np.empty(ng(self.nc))
        lib().orc_plaquette(self.pp, _p(self.Unext if t else self.U), C.c_long(index), d1, d2, o1, o2, _p(out))
        return out

    def get_b(self, index, d, t=0):
        out = np.empty(na(self.nc))
        lib().orc_get_b(self.pp, _p(self.Unext if t else self.U), C.c_long(index), d, _p(out))
        return out

    def gauss_constraint(self, index):
        out = np.empty(na(self.nc))
        lib().orc_gauss_constraint(self.pp, _p(self.U), _p(self.E), _p(self.rho), C.c_long(index), _p(out))
        return out

    def projected_poynting(self, d):
        out = np.empty(2 * self.dims[d])
        rc = lib().orc_projected_poynting(self.pp, _p(self.U), _p(self.Unext), _p(self.E), d, _p(out))
        if rc != 0:
            raise ValueError("Poynting vector: SU(2) only")
        return out.reshape(2, self.dims[d])

    def gauss_field(self):
        out = np.empty((self.V, na(self.nc)))
        lib().orc_gauss_field(self.pp, _p(self.U), _p(self.E), _p(self.rho), _p(out))
        return out

    # physics/fields/FastTYMSolver.java
    def update_links(self):
        lib().orc_update_links(self.pp, _p(self.U), _p(self.E), _p(self.Unext), _p(self.active))

    def update_grid(self):
        lib().orc_update_grid(self.pp, _p(self.U), _p(self.E), _p(self.J), _p(self.Unext), _p(self.active))

    def update_grid_tym(self):
        """TemporalYangMillsSolver.step (the plaquette form) in place of update_grid."""
        lib().orc_update_grid_tym(self.pp, _p(self.U), _p(self.E), _p(self.J), _p(self.Unext), _p(self.active))

    def update_grid_implicit(self, iterations, damping):
        """ImplicitTYMSolver.step (SU(2), SU(3)) in place of update_grid."""
        rc = lib().orc_implicit_update_grid(self.pp, _p(self.U), _p(self.E), _p(self.J), _p(self.Unext),
                                            _p(self.active), int(iterations), C.c_double(damping))
        if rc != 0:
            raise ValueError("implicit solver: SU(2) only")

    def update_grid_omp(self, nthreads):
        lib().orc_update_grid_omp(self.pp, _p(self.U), _p(self.E), _p(self.J), _p(self.Unext),
                                  _p(self.active), int(nthreads))

    def update_grid_range_omp(self, s0, s1, nthreads):
        lib().orc_update_grid_range_omp(self.pp, _p(self.U), _p(self.E), _p(self.J), _p(self.Unext),
                                        _p(self.active), C.c_long(s0), C.c_long(s1), int(nthreads))

    def store_fields(self):
        # Cell.reassignLinks: swap U and Unext (physics/grid/Cell.java:173-177)
        self.U, self.Unext = self.Unext, self.U

    # measurements
    def bulk(self):
        out = np.empty(13)
        lib().orc_bulk(self.pp, _p(self.U), _p(self.Unext), _p(self.E), _p(self.rho), _p(self.eval), _p(out))
        return out

    def energy_density(self):
        out = np.empty(self.V)
        lib().orc_energy_density(self.pp, _p(self.U), _p(self.Unext), _p(self.E), _p(self.eval), _p(out))
        return out

    def projected_energy(self, d):
        out = np.empty(4 * self.dims[d])
        lib().orc_projected_energy(self.pp, _p(self.U), _p(self.Unext), _p(self.E), _p(self.eval), d, _p(out))
        return out.reshape(4, self.dims[d])

    # seeded initial conditions
    def random_links(self, seed, sigma, stream=0):
        """U_i(x) = getLink(A_i(x)), A_i^a(x) ~ N(0, sigma^2) per generator component."""
        k = ngen(self.nc)
        gen = random_gen(seed, stream, self.V * 3 * k, sigma).reshape(self.V * 3, k)
        L = lib()
        U = self.U.reshape(self.V * 3, ng(self.nc))
        tmp = np.empty(na(self.nc))
        for m in range(self.V * 3):
            L.orc_gen_to_alg(self.nc, _p(gen[m]), _p(tmp))
            L.orc_alg_getlink(self.nc, _p(tmp), _p(U[m]))

    def random_fields(self, seed, sigma_a, sigma_e):
        """random_links(seed, sigma_a) and random_e(seed, sigma_e) in one C loop."""
        lib().orc_random_fields(self.pp, C.c_uint64(seed), C.c_double(sigma_a), C.c_double(sigma_e),
                                _p(self.U), _p(self.E))

    def random_e(self, seed, sigma, stream=1):
        k = ngen(self.nc)
        gen = random_gen(seed, stream, self.V * 3 * k, sigma).reshape(self.V * 3, k)
        L = lib()
        E = self.E.reshape(self.V * 3, na(self.nc))
        for m in range(self.V * 3):
            L.orc_gen_to_alg(self.nc, _p(gen[m]), _p(E[m]))

    def gauss_project(self, tol_g2=1e-26, maxit=5000):
        g2 = C.c_double()
        dp = C.POINTER(C.c_double)
        it = lib().orc_gauss_project_cg(self.pp, self.U.ctypes.data_as(dp), self.E.ctypes.data_as(dp),
                                        self.rho.ctypes.data_as(dp), tol_g2, maxit, C.byref(g2))
        return it, g2.value

    def gauss_restoration(self, gamma, maxit, absval):
        v = C.c_double()
        dp = C.POINTER(C.c_double)
        it = lib().orc_gauss_restoration(self.pp, self.U.ctypes.data_as(dp), self.Unext.ctypes.data_as(dp),
                                         self.E.ctypes.data_as(dp), self.rho.ctypes.data_as(dp),
                                         gamma, maxit, absval, C.byref(v))
        return it, v.value

    # generator-component views (the device storage basis)
    def e_gen(self):
        out = np.empty((self.V, 3, ngen(self.nc)))
        L = lib()
        E = self.E.reshape(-1, na(self.nc))
        O = out.reshape(-1, ngen(self.nc))
        for m in range(E.shape[0]):
            L.orc_alg_to_gen(self.nc, _p(E[m]), _p(O[m]))
        return out


class OracleParticles:
    """CGC particle list (physics/particles/CGCParticle.java) as arrays."""

    def __init__(self, nc, n):
        self.nc = nc
        self.n = int(n)
        self.pos0 = np.zeros((n, 3))
        self.pos1 = np.zeros((n, 3))
        self.vel = np.zeros((n, 3))
        self.Q0 = np.zeros((n, na(nc)))
        self.Q1 = np.zeros((n, na(nc)))
        self.dir = np.zeros(n, np.int32)
        self.flag = np.zeros(n, np.uint8)
        self.Ulink = np.zeros((n, ng(nc)))

    def copy(self):
        o = OracleParticles(self.nc, self.n)
        for k in ("pos0", "pos1", "vel", "Q0", "Q1", "dir", "flag", "Ulink"):
            setattr(o, k, getattr(self, k).copy())
        return o

    def ngp(self, grid, pos):
        out = np.empty((pos.shape[0], 3), np.int32)
        for k in range(pos.shape[0]):
            lib().orc_ngp(grid.pp, _p(np.ascontiguousarray(pos[k])), _p(out[k]))
        return out


class OracleSimulation:
    """Phase order of physics/Simulation.java (initialize :318-352, step :373-435)."""

    def __init__(self, grid, particles=None, implicit=None):
        self.grid = grid
        self.particles = particles
        self.steps = 0
        self.implicit = implicit  # (iterations, damping) for ImplicitTYMSolver

    def _cpic_phases(self):
        g, P, L = self.grid, self.particles, lib()
        if P is None or P.n == 0:
            return
        # 6) rho from particle positions (resetCharge + interpolateChargedensity)
        g.rho[...] = 0.0
        L.orc_cpic_charge_density(g.pp, C.c_long(P.n), _p(P.pos0), _p(P.Q0), _p(g.rho))
        # 8) positions
        L.orc_cpic_update_positions(g.pp, C.c_long(P.n), _p(P.pos0), _p(P.pos1), _p(P.vel))
        # 9) parallel transporters
        L.orc_cpic_to_particle(g.pp, C.c_long(P.n), _p(P.pos0), _p(P.pos1), _p(P.vel), _p(P.dir),
                               _p(g.Unext), _p(P.Ulink), _p(P.flag))
        # 10) charges
        L.orc_cpic_update_charges(g.nc, C.c_long(P.n), _p(P.Q0), _p(P.Q1), _p(P.Ulink), _p(P.flag))
        # 11) currents
        g.J[...] = 0.0
        L.orc_cpic_to_grid(g.pp, C.c_long(P.n), _p(P.pos0), _p(P.pos1), _p(P.vel), _p(P.dir),
                           _p(P.Q0), _p(P.Q1), _p(g.J))

    def initialize(self):
        self.grid.update_links()
        self._cpic_phases()

    def step(self):
        self.steps += 1
        P = self.particles
        if P is not None and P.n:
            lib().orc_cpic_reassign(self.grid.nc, C.c_long(P.n), _p(P.pos0), _p(P.pos1), _p(P.Q0), _p(P.Q1))
        self.grid.store_fields()
        if self.implicit is not None:
            self.grid.update_grid_implicit(*self.implicit)
        else:
            self.grid.update_grid()
        self._cpic_phases()
