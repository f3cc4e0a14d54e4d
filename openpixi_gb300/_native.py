"""ctypes binding of libopixi_gpu.so (the C ABI declared in include/opixi.h).

The library is built in-tree by ``openpixi_gb300.build`` (``__graft_entry__.build()``
does it).  Loading fails loudly when it is missing: there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libopixi_gpu.so")

OPX_OK = 0
OPX_ERR_INVALID = -1
OPX_ERR_CUDA = -2
OPX_ERR_NOMEM = -3
OPX_ERR_NUMERIC = -4
OPX_ERR_UNSUPPORTED = -5
OPX_ERR_TIMEOUT = -6

OPX_F64 = 0
OPX_F32 = 1

FIELD_U, FIELD_UNEXT, FIELD_E, FIELD_J, FIELD_RHO = range(5)
LAYOUT_REF, LAYOUT_GEN = 0, 1
PHASE_EOM, PHASE_CPIC, PHASE_DIA, PHASE_LINKS = range(4)
SOLVER_FAST, SOLVER_IMPLICIT = 0, 1
NUM_PHASES = 4

# Every symbol include/opixi.h declares (checked by the CPU test suite).
EXPORTED = [
    "opx_create", "opx_destroy", "opx_last_error", "opx_version",
    "opx_upload", "opx_download", "opx_set_active", "opx_set_evaluatable",
    "opx_step_links", "opx_update_grid", "opx_store_fields", "opx_initialize", "opx_step",
    "opx_reunitarize", "opx_synchronize", "opx_steps_done",
    "opx_reduce", "opx_energy_density", "opx_projected_energy", "opx_gauss_field",
    "opx_particles_upload", "opx_particles_download", "opx_cpic_phases",
    "opx_init_random", "opx_gauss_project",
    "opx_set_profiling", "opx_phase_times", "opx_time_steps", "opx_kernel_launches",
    "opx_host_alloc", "opx_host_free", "opx_reduce_noalloc",
    "opx_objective_value", "opx_objective_tangent", "opx_objective_gradient",
    "opx_batch_create", "opx_batch_destroy", "opx_batch_last_error", "opx_batch_init_random",
    "opx_batch_upload", "opx_batch_download", "opx_batch_initialize", "opx_batch_autotune",
    "opx_batch_set_schedule",
    "opx_batch_run", "opx_batch_time_run", "opx_batch_reduce", "opx_batch_config",
    "opx_batch_kernel_launches",
    "opx_energy_objective", "opx_energy_tangent", "opx_energy_gradient", "opx_cgc_mv",
    "opx_particles_count", "opx_projected_poynting", "opx_cgc_mv_super", "opx_super_groups",
    "opx_super_download", "opx_super_upload", "opx_occupation_numbers", "opx_set_field_solver",
    "opx_cgc_wilson_lines", "opx_occupation_numbers_ex", "opx_step_measured",
]


class OpixiError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"opixi error {code}: {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [("ncolors", C.c_int), ("dims", C.c_int * 3), ("a", C.c_double * 3),
                ("dt", C.c_double), ("g", C.c_double), ("precision", C.c_int),
                ("reunit_every", C.c_int), ("device", C.c_int), ("flags", C.c_int)]


class Observables(C.Structure):
    _fields_ = [("e2", C.c_double * 3), ("b2", C.c_double * 3), ("px", C.c_double),
                ("py", C.c_double), ("pz", C.c_double), ("gauss", C.c_double),
                ("rho2", C.c_double), ("e2_total", C.c_double), ("b2_total", C.c_double)]

    def as_dict(self):
        return {"e2": list(self.e2), "b2": list(self.b2), "px": self.px, "py": self.py, "pz": self.pz,
                "gauss": self.gauss, "rho2": self.rho2, "e2_total": self.e2_total,
                "b2_total": self.b2_total}


class MVNucleus(C.Structure):
    _fields_ = [("direction", C.c_int), ("orientation", C.c_int), ("location", C.c_double),
                ("width", C.c_double), ("mu", C.c_double), ("use_seed", C.c_int), ("seed", C.c_int),
                ("uvt", C.c_double), ("coherence", C.c_double), ("ir", C.c_double)]


class Particles(C.Structure):
    _fields_ = [("n", C.c_long), ("pos0", C.c_void_p), ("pos1", C.c_void_p), ("vel", C.c_void_p),
                ("Q0", C.c_void_p), ("Q1", C.c_void_p), ("dir", C.c_void_p),
                ("update_charge", C.c_void_p)]


_lib = None


OBJ_ENERGY, OBJ_ANISOTROPY = 0, 1
WRT_E, WRT_RHO = 0, 1


class Objective(C.Structure):
    """opx_objective: objective kind, longitudinal direction, box of cells."""
    _fields_ = [("kind", C.c_int), ("direction", C.c_int), ("lo", C.c_int * 3), ("hi", C.c_int * 3)]


def load(path=None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"libopixi_gpu.so not built ({p}); run openpixi_gb300.build.build()")
    L = C.CDLL(p)
    vp, sz, dp = C.c_void_p, C.c_size_t, C.POINTER(C.c_double)
    sig = {
        "opx_create": (C.c_int, [C.POINTER(Config), C.POINTER(vp)]),
        "opx_destroy": (None, [vp]),
        "opx_last_error": (C.c_char_p, [vp]),
        "opx_version": (C.c_int, []),
        "opx_upload": (C.c_int, [vp, C.c_int, vp, sz, C.c_int]),
        "opx_download": (C.c_int, [vp, C.c_int, vp, sz, C.c_int]),
        "opx_set_active": (C.c_int, [vp, vp, sz]),
        "opx_set_evaluatable": (C.c_int, [vp, vp, sz]),
        "opx_step_links": (C.c_int, [vp]),
        "opx_update_grid": (C.c_int, [vp]),
        "opx_store_fields": (C.c_int, [vp]),
        "opx_initialize": (C.c_int, [vp]),
        "opx_step": (C.c_int, [vp, C.c_int]),
        "opx_reunitarize": (C.c_int, [vp]),
        "opx_synchronize": (C.c_int, [vp]),
        "opx_steps_done": (C.c_long, [vp]),
        "opx_reduce": (C.c_int, [vp, C.POINTER(Observables)]),
        "opx_step_measured": (C.c_int, [vp, C.c_int, C.POINTER(Observables)]),
        "opx_energy_density": (C.c_int, [vp, vp, sz]),
        "opx_projected_energy": (C.c_int, [vp, C.c_int, vp, sz]),
        "opx_gauss_field": (C.c_int, [vp, vp, sz]),
        "opx_particles_upload": (C.c_int, [vp, C.POINTER(Particles)]),
        "opx_particles_download": (C.c_int, [vp, C.POINTER(Particles)]),
        "opx_cpic_phases": (C.c_int, [vp, C.c_int]),
        "opx_init_random": (C.c_int, [vp, C.c_uint64, C.c_double, C.c_double]),
        "opx_gauss_project": (C.c_int, [vp, C.c_double, C.c_int, C.POINTER(C.c_int), dp]),
        "opx_set_profiling": (C.c_int, [vp, C.c_int]),
        "opx_phase_times": (C.c_int, [vp, dp, C.POINTER(C.c_long), C.c_int]),
        "opx_time_steps": (C.c_int, [vp, C.c_int, dp]),
        "opx_kernel_launches": (C.c_long, [vp]),
        "opx_host_alloc": (vp, [sz]),
        "opx_host_free": (None, [vp]),
        "opx_batch_create": (C.c_int, [C.c_int, C.c_int, vp, vp, C.c_double, C.c_double, C.c_int, C.c_int,
                                       C.c_int, C.POINTER(vp)]),
        "opx_batch_destroy": (None, [vp]),
        "opx_batch_last_error": (C.c_char_p, [vp]),
        "opx_batch_init_random": (C.c_int, [vp, vp, C.c_double, C.c_double, C.c_double]),
        "opx_batch_upload": (C.c_int, [vp, C.c_int, C.c_int, vp, sz, C.c_int]),
        "opx_batch_download": (C.c_int, [vp, C.c_int, C.c_int, vp, sz, C.c_int]),
        "opx_batch_initialize": (C.c_int, [vp]),
        "opx_batch_autotune": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "opx_batch_set_schedule": (C.c_int, [vp, C.c_int, C.c_int]),
        "opx_batch_run": (C.c_int, [vp, C.c_int, C.c_int]),
        "opx_batch_time_run": (C.c_int, [vp, C.c_int, C.c_int, dp]),
        "opx_batch_reduce": (C.c_int, [vp, vp]),
        "opx_batch_config": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "opx_batch_kernel_launches": (C.c_long, [vp]),
        "opx_cgc_mv": (C.c_int, [vp, vp, C.c_int]),
        "opx_cgc_wilson_lines": (C.c_int, [vp, C.c_int, dp, dp, C.c_size_t, dp]),
        "opx_particles_count": (C.c_long, [vp]),
        "opx_projected_poynting": (C.c_int, [vp, C.c_int, vp, C.c_size_t]),
        "opx_cgc_mv_super": (C.c_int, [vp, vp, C.c_int]),
        "opx_super_groups": (C.c_int, [vp]),
        "opx_super_download": (C.c_int, [vp, C.c_int, vp, vp, vp, vp, C.c_size_t]),
        "opx_super_upload": (C.c_int, [vp, C.c_int, C.c_long, C.c_long, vp]),
        "opx_occupation_numbers": (C.c_int, [vp, C.c_int, C.c_double, vp, C.c_size_t, vp, vp, vp]),
        "opx_occupation_numbers_ex": (C.c_int, [vp, vp, C.c_int, C.c_double, vp, C.c_size_t, vp, vp, vp]),
        "opx_set_field_solver": (C.c_int, [vp, C.c_int, C.c_int, C.c_double]),
        "opx_energy_objective": (C.c_int, [vp, C.c_int, vp, vp, vp, C.c_double, dp]),
        "opx_energy_tangent": (C.c_int, [vp, C.c_int, vp, vp, vp, dp, dp]),
        "opx_energy_gradient": (C.c_int, [vp, C.c_int, C.c_int, vp, vp, dp, vp, sz]),
        "opx_objective_value": (C.c_int, [vp, C.POINTER(Objective), C.c_int, vp, vp, C.c_double, dp]),
        "opx_objective_tangent": (C.c_int, [vp, C.POINTER(Objective), C.c_int, vp, vp, dp, dp]),
        "opx_objective_gradient": (C.c_int, [vp, C.POINTER(Objective), C.c_int, C.c_int, C.c_int, dp, vp, sz]),
        "opx_reduce_noalloc": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                         C.c_double, vp, vp, vp, vp, vp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def ptr(a):
    if a is None:
        return None
    assert isinstance(a, np.ndarray) and a.flags["C_CONTIGUOUS"], "C-contiguous numpy array required"
    return a.ctypes.data_as(C.c_void_p)


WINDOW_GAUSSIAN, WINDOW_TUKEY, WINDOW_CONE = 1, 2, 4


class OccupationOptions(C.Structure):
    """opx_occupation_options (include/opixi.h)."""
    _fields_ = [("mirrored_direction", C.c_int), ("windows", C.c_int), ("collision_time", C.c_double),
                ("collision_position", C.c_double * 3), ("cone_velocity", C.c_double * 3),
                ("tukey_width", C.c_double)]


class Handle:
    """Owning wrapper around one ``opx_ctx`` (one lattice on one GPU)."""

    def __init__(self, ncolors, dims, a=(1.0, 1.0, 1.0), dt=0.05, g=1.0, precision=OPX_F64,
                 reunit_every=0, device=0):
        self.L = load()
        if np.ndim(a) == 0:
            a = (float(a),) * 3
        cfg = Config(int(ncolors), (C.c_int * 3)(*[int(d) for d in dims]), (C.c_double * 3)(*a),
                     float(dt), float(g), int(precision), int(reunit_every), int(device), 0)
        h = C.c_void_p()
        rc = self.L.opx_create(C.byref(cfg), C.byref(h))
        if rc != OPX_OK:
            raise OpixiError(rc, self.L.opx_last_error(None).decode())
        self.h = h
        self.ncolors = int(ncolors)
        self.a = tuple(float(x) for x in a)
        self.dt = float(dt)
        self.dims = tuple(int(d) for d in dims)
        self.V = int(np.prod(self.dims))
        self.precision = precision
        self.ng = 18 if ncolors == 3 else 4
        self.na_ref = 9 if ncolors == 3 else 3
        self.ngen = 8 if ncolors == 3 else 3

    def close(self):
        if getattr(self, "h", None):
            self.L.opx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc):
        if rc != OPX_OK:
            raise OpixiError(rc, self.L.opx_last_error(self.h).decode())
        return rc

    # ---- transfers ----
    def _shape(self, field, layout):
        na = self.na_ref if layout == LAYOUT_REF else self.ngen
        if field in (FIELD_U, FIELD_UNEXT):
            return (self.V, 3, self.ng)
        if field in (FIELD_E, FIELD_J):
            return (self.V, 3, na)
        return (self.V, na)

    def upload(self, field, arr, layout=LAYOUT_REF):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self.check(self.L.opx_upload(self.h, field, ptr(a), a.size, layout))

    def download(self, field, layout=LAYOUT_REF, out=None):
        shp = self._shape(field, layout)
        out = np.empty(shp) if out is None else out
        self.check(self.L.opx_download(self.h, field, ptr(out), out.size, layout))
        return out

    def set_active(self, mask):
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        self.check(self.L.opx_set_active(self.h, ptr(m), 0 if m is None else m.size))

    def set_evaluatable(self, mask):
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        self.check(self.L.opx_set_evaluatable(self.h, ptr(m), 0 if m is None else m.size))

    # ---- solver ----
    def step_links(self):
        self.check(self.L.opx_step_links(self.h))

    def update_grid(self):
        self.check(self.L.opx_update_grid(self.h))

    def store_fields(self):
        self.check(self.L.opx_store_fields(self.h))

    def initialize(self):
        self.check(self.L.opx_initialize(self.h))

    def step(self, n=1):
        self.check(self.L.opx_step(self.h, int(n)))

    def reunitarize(self):
        self.check(self.L.opx_reunitarize(self.h))

    def synchronize(self):
        self.check(self.L.opx_synchronize(self.h))

    @property
    def steps_done(self):
        return self.L.opx_steps_done(self.h)

    # ---- reductions ----
    def reduce(self):
        o = Observables()
        self.check(self.L.opx_reduce(self.h, C.byref(o)))
        return o

    def step_measured(self, n):
        """n steps with BulkQuantities after each: a list of n Observables (what
        reduce() returns after each step)."""
        out = (Observables * max(int(n), 1))()
        self.check(self.L.opx_step_measured(self.h, int(n), out))
        return list(out)[:max(int(n), 0)]

    def energy_density(self):
        out = np.empty(self.V)
        self.check(self.L.opx_energy_density(self.h, ptr(out), out.size))
        return out

    def projected_energy(self, d):
        # an invalid direction is passed through so that the library reports it
        out = np.empty(4 * self.dims[d] if 0 <= int(d) < 3 else 1)
        self.check(self.L.opx_projected_energy(self.h, int(d), ptr(out), out.size))
        return out.reshape(4, self.dims[d])

    def projected_poynting(self, d):
        out = np.empty(2 * self.dims[d] if 0 <= int(d) < 3 else 1)
        self.check(self.L.opx_projected_poynting(self.h, int(d), ptr(out), out.size))
        return out.reshape(2, self.dims[d])

    def gauss_field(self):
        out = np.empty((self.V, self.ngen))
        self.check(self.L.opx_gauss_field(self.h, ptr(out), out.size))
        return out

    # ---- particles ----
    def particles_upload(self, pos0, pos1, vel, Q0, Q1, direction):
        arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (pos0, pos1, vel, Q0, Q1)]
        d = np.ascontiguousarray(direction, dtype=np.int32)
        self._pkeep = arrs + [d]
        p = Particles(len(d), *[ptr(x) for x in arrs], ptr(d), None)
        self.check(self.L.opx_particles_upload(self.h, C.byref(p)))
        self.np = len(d)

    def particles_download(self):
        n = self.np
        out = {k: np.empty((n, 3)) for k in ("pos0", "pos1", "vel")}
        out["Q0"] = np.empty((n, self.na_ref))
        out["Q1"] = np.empty((n, self.na_ref))
        out["dir"] = np.empty(n, np.int32)
        out["update_charge"] = np.empty(n, np.uint8)
        p = Particles(n, ptr(out["pos0"]), ptr(out["pos1"]), ptr(out["vel"]), ptr(out["Q0"]),
                      ptr(out["Q1"]), ptr(out["dir"]), ptr(out["update_charge"]))
        self.check(self.L.opx_particles_download(self.h, C.byref(p)))
        return out

    def cpic_phases(self, reassign=True):
        self.check(self.L.opx_cpic_phases(self.h, 1 if reassign else 0))

    # ---- initial conditions ----
    def init_random(self, seed, sigma_a, sigma_e):
        self.check(self.L.opx_init_random(self.h, C.c_uint64(seed), float(sigma_a), float(sigma_e)))

    def gauss_project(self, tol=1e-26, maxit=5000):
        it = C.c_int()
        g2 = C.c_double()
        self.check(self.L.opx_gauss_project(self.h, float(tol), int(maxit), C.byref(it), C.byref(g2)))
        return it.value, g2.value

    # ---- CGC initial conditions ----
    def cgc_mv(self, nuclei):
        """nuclei: list of dicts with the MVNucleus fields."""
        arr = (MVNucleus * len(nuclei))()
        for k, nu in enumerate(nuclei):
            for f, _ in MVNucleus._fields_:
                setattr(arr[k], f, nu[f])
        self.check(self.L.opx_cgc_mv(self.h, arr, len(nuclei)))
        self.np = self.L.opx_particles_count(self.h)

    def cgc_wilson_lines(self, nucleus=0, dipole=True):
        """WilsonLineObservables of nucleus k of the last CGC call: (tadpole,
        dipole bins or None, bin width)."""
        import math
        n1, n2 = self.dims[1], self.dims[2]
        nb = int(math.sqrt(n1 * n2)) // 2  # (int) Math.sqrt(totalCells) / 2
        t, w = C.c_double(), C.c_double()
        d = np.empty(nb) if dipole else None
        self.check(self.L.opx_cgc_wilson_lines(self.h, int(nucleus), C.byref(t),
                                               None if d is None else d.ctypes.data_as(C.POINTER(C.c_double)),
                                               nb if dipole else 0, C.byref(w)))
        return t.value, d, w.value

    def set_field_solver(self, kind, iterations=0, damping=0.0):
        """FastTYMSolver (SOLVER_FAST) or ImplicitTYMSolver(iterations, damping) (SOLVER_IMPLICIT)."""
        self.check(self.L.opx_set_field_solver(self.h, int(kind), int(iterations), float(damping)))

    def occupation_numbers(self, max_iter=100, accuracy_goal=1e-18, with_n=True, mirrored_direction=-1,
                           windows=0, collision_time=0.0, collision_position=(0.0, 0.0, 0.0),
                           cone_velocity=(0.0, 0.0, 0.0), tukey_width=0.0):
        """OccupationNumbersInTime: (n [V][3] or None, energy density, iterations,
        last divergence); the mirrored grid and the windows (WINDOW_* flags) as
        the diagnostic's options."""
        n = np.empty((self.V, self.ngen)) if with_n else None
        e, it, dv = C.c_double(), C.c_int(), C.c_double()
        opt = OccupationOptions(int(mirrored_direction), int(windows), float(collision_time),
                                (C.c_double * 3)(*collision_position), (C.c_double * 3)(*cone_velocity),
                                float(tukey_width))
        self.check(self.L.opx_occupation_numbers_ex(self.h, C.byref(opt), int(max_iter), float(accuracy_goal),
                                                    ptr(n), 0 if n is None else n.size, C.byref(e), C.byref(it),
                                                    C.byref(dv)))
        return n, e.value, it.value, dv.value

    # ---- super particles (temporal optimized cgc ngp) ----
    def cgc_mv_super(self, nuclei):
        arr = (MVNucleus * len(nuclei))()
        for k, nu in enumerate(nuclei):
            for f, _ in MVNucleus._fields_:
                setattr(arr[k], f, nu[f])
        self.check(self.L.opx_cgc_mv_super(self.h, arr, len(nuclei)))

    @property
    def super_groups(self):
        return self.L.opx_super_groups(self.h)

    def super_download(self, g):
        o, n, b = C.c_int(), C.c_long(), C.c_long()
        self.check(self.L.opx_super_download(self.h, int(g), C.byref(o), C.byref(n), C.byref(b), None, 0))
        from .diagnostics import java_round
        ppc = java_round(self.a[0] / self.dt)  # LightConeNGPParticleCreator.java:89
        Q = np.empty((ppc, n.value, self.na_ref))
        self.check(self.L.opx_super_download(self.h, int(g), None, None, None, ptr(Q), Q.size))
        return {"orientation": o.value, "n": n.value, "base": b.value, "Q": Q}

    def super_upload(self, orientation, n, base, Q):
        q = np.ascontiguousarray(Q, dtype=np.float64)
        self.check(self.L.opx_super_upload(self.h, int(orientation), int(n), int(base), ptr(q) if q.size else None))

    # ---- differentiation form (SU(2)) ----
    @staticmethod
    def _box(lo, hi):
        lo_c = None if lo is None else (C.c_int * 3)(*[int(v) for v in lo])
        hi_c = None if hi is None else (C.c_int * 3)(*[int(v) for v in hi])
        return lo_c, hi_c

    def energy_objective(self, nsteps, lo=None, hi=None, dE=None, h=0.0):
        lo_c, hi_c = self._box(lo, hi)
        d = None if dE is None else np.ascontiguousarray(dE, dtype=np.float64)
        J = C.c_double()
        self.check(self.L.opx_energy_objective(self.h, int(nsteps), lo_c, hi_c, ptr(d), float(h), C.byref(J)))
        return J.value

    def energy_tangent(self, nsteps, dE, lo=None, hi=None):
        lo_c, hi_c = self._box(lo, hi)
        d = np.ascontiguousarray(dE, dtype=np.float64)
        J, dJ = C.c_double(), C.c_double()
        self.check(self.L.opx_energy_tangent(self.h, int(nsteps), lo_c, hi_c, ptr(d), C.byref(J), C.byref(dJ)))
        return J.value, dJ.value

    def energy_gradient(self, nsteps, ckpt, lo=None, hi=None):
        lo_c, hi_c = self._box(lo, hi)
        g = np.empty((self.V, 3, self.ngen))
        J = C.c_double()
        self.check(self.L.opx_energy_gradient(self.h, int(nsteps), int(ckpt), lo_c, hi_c, C.byref(J), ptr(g), g.size))
        return J.value, g

    def _objective(self, kind, direction, lo, hi):
        lo = (0, 0, 0) if lo is None else lo
        hi = tuple(d - 1 for d in self.dims) if hi is None else hi
        return Objective(int(kind), int(direction), (C.c_int * 3)(*[int(v) for v in lo]),
                         (C.c_int * 3)(*[int(v) for v in hi]))

    def objective_value(self, nsteps, kind=OBJ_ENERGY, direction=0, lo=None, hi=None, dE=None, drho=None, h=0.0):
        """J of the objective after nsteps, with E_0 moved by h (dE + divT K^+ drho)."""
        ob = self._objective(kind, direction, lo, hi)
        d = None if dE is None else np.ascontiguousarray(dE, dtype=np.float64)
        r = None if drho is None else np.ascontiguousarray(drho, dtype=np.float64)
        J = C.c_double()
        self.check(self.L.opx_objective_value(self.h, C.byref(ob), int(nsteps), ptr(d), ptr(r), float(h),
                                              C.byref(J)))
        return J.value

    def objective_tangent(self, nsteps, kind=OBJ_ENERGY, direction=0, lo=None, hi=None, dE=None, drho=None):
        ob = self._objective(kind, direction, lo, hi)
        d = None if dE is None else np.ascontiguousarray(dE, dtype=np.float64)
        r = None if drho is None else np.ascontiguousarray(drho, dtype=np.float64)
        J, dJ = C.c_double(), C.c_double()
        self.check(self.L.opx_objective_tangent(self.h, C.byref(ob), int(nsteps), ptr(d), ptr(r), C.byref(J),
                                                C.byref(dJ)))
        return J.value, dJ.value

    def objective_gradient(self, nsteps, ckpt, kind=OBJ_ENERGY, direction=0, lo=None, hi=None, wrt=WRT_E):
        """(J, dJ/dE_0 [V][3][ngen]) or (J, dJ/drho [V][ngen])."""
        ob = self._objective(kind, direction, lo, hi)
        g = np.empty((self.V, 3, self.ngen)) if wrt == WRT_E else np.empty((self.V, self.ngen))
        J = C.c_double()
        self.check(self.L.opx_objective_gradient(self.h, C.byref(ob), int(nsteps), int(ckpt), int(wrt), C.byref(J),
                                                 ptr(g), g.size))
        return J.value, g

    # ---- timing ----
    def set_profiling(self, on=True):
        self.check(self.L.opx_set_profiling(self.h, 1 if on else 0))

    def phase_times(self):
        ms = (C.c_double * NUM_PHASES)()
        n = (C.c_long * NUM_PHASES)()
        self.check(self.L.opx_phase_times(self.h, ms, n, NUM_PHASES))
        return list(ms), list(n)

    def time_steps(self, n):
        ms = C.c_double()
        self.check(self.L.opx_time_steps(self.h, int(n), C.byref(ms)))
        return ms.value

    @property
    def kernel_launches(self):
        return self.L.opx_kernel_launches(self.h)


class Batch:
    """Owning wrapper around one ``opx_batch`` (many independent lattices)."""

    def __init__(self, ncolors, dims_list, dt=0.05, g=1.0, precision=OPX_F32, reunit_every=0, device=0,
                 spacings=None):
        self.L = load()
        dims = np.ascontiguousarray(np.asarray(dims_list, dtype=np.int32).reshape(-1, 3))
        a = None if spacings is None else np.ascontiguousarray(np.asarray(spacings, float).reshape(-1, 3))
        h = C.c_void_p()
        rc = self.L.opx_batch_create(int(ncolors), dims.shape[0], ptr(dims), ptr(a), float(dt), float(g),
                                     int(precision), int(reunit_every), int(device), C.byref(h))
        if rc != OPX_OK:
            raise OpixiError(rc, "opx_batch_create failed")
        self.h = h
        self.ncolors = int(ncolors)
        self.dims = [tuple(int(x) for x in d) for d in dims]
        self.n = dims.shape[0]
        self.ng = 18 if ncolors == 3 else 4
        self.na_ref = 9 if ncolors == 3 else 3
        self.ngen = 8 if ncolors == 3 else 3

    def close(self):
        if getattr(self, "h", None):
            self.L.opx_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc):
        if rc != OPX_OK:
            raise OpixiError(rc, self.L.opx_batch_last_error(self.h).decode())
        return rc

    def init_random(self, seeds, sigma_a, sigma_e, tol=1e-24):
        s = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64))
        self.check(self.L.opx_batch_init_random(self.h, ptr(s), float(sigma_a), float(sigma_e), float(tol)))

    def _shape(self, q, field, layout):
        V = int(np.prod(self.dims[q]))
        na = self.na_ref if layout == LAYOUT_REF else self.ngen
        return (V, 3, self.ng) if field in (FIELD_U, FIELD_UNEXT) else (V, 3, na)

    def upload(self, q, field, arr, layout=LAYOUT_REF):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self.check(self.L.opx_batch_upload(self.h, int(q), field, ptr(a), a.size, layout))

    def download(self, q, field, layout=LAYOUT_REF):
        out = np.empty(self._shape(q, field, layout))
        self.check(self.L.opx_batch_download(self.h, int(q), field, ptr(out), out.size, layout))
        return out

    def initialize(self):
        self.check(self.L.opx_batch_initialize(self.h))

    def autotune(self, steps=5):
        c, b = C.c_int(), C.c_int()
        self.check(self.L.opx_batch_autotune(self.h, int(steps), C.byref(c), C.byref(b)))
        return c.value, b.value

    def set_schedule(self, cluster, block):
        """cluster 0: one launch per step over all events; 1-8: persistent clusters."""
        self.check(self.L.opx_batch_set_schedule(self.h, int(cluster), int(block)))

    def run(self, nsteps, use_graph=True):
        self.check(self.L.opx_batch_run(self.h, int(nsteps), 1 if use_graph else 0))

    def time_run(self, nsteps, use_graph=True):
        ms = C.c_double()
        self.check(self.L.opx_batch_time_run(self.h, int(nsteps), 1 if use_graph else 0, C.byref(ms)))
        return ms.value

    def reduce(self):
        out = (Observables * self.n)()
        self.check(self.L.opx_batch_reduce(self.h, out))
        return list(out)

    def config(self):
        c, b, n = C.c_int(), C.c_int(), C.c_int()
        self.check(self.L.opx_batch_config(self.h, C.byref(c), C.byref(b), C.byref(n)))
        return {"cluster": c.value, "block": b.value, "clusters": n.value}

    @property
    def kernel_launches(self):
        return self.L.opx_batch_kernel_launches(self.h)


class PinnedArray:
    """numpy view of page-locked host memory from opx_host_alloc."""

    def __init__(self, shape, dtype=np.float64):
        self.L = load()
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.p = self.L.opx_host_alloc(n)
        if not self.p:
            raise MemoryError("opx_host_alloc failed")
        buf = (C.c_char * n).from_address(self.p)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self.p:
            self.array = None
            self.L.opx_host_free(self.p)
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
