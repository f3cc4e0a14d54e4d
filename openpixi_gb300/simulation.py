"""Simulation, Grid and FieldSolver: the host-side mirror of the reference's Java
API for this path, backed by one libopixi_gpu handle.

  Simulation      physics/Simulation.java (ctor :185-281, initialize :318-352,
                  step :373-435, continues :441-443, run :448-452)
  Grid            physics/grid/Grid.java (device-resident; bulk accessors plus
                  per-cell getters that read a host mirror refreshed on demand)
  FastTYMSolver   physics/fields/FastTYMSolver.java (step / stepLinks on the GPU)

The fields live on the GPU between steps; the host mirror is read only when a
caller asks for per-cell values (getU, getE, ...), which is the one explicit
synchronisation point.
"""
import numpy as np

from . import _native as N
from .settings import SUPPORTED


class FieldSolver:
    """physics/fields/FieldSolver.java:114-156 (the plug-in the Grid calls)."""

    def step(self, grid, time_step):
        raise NotImplementedError

    def stepLinks(self, grid, time_step):
        raise NotImplementedError

    def clone(self):
        return type(self)()


class FastTYMSolver(FieldSolver):
    """FastTYMSolver.CombinedUpdate / UpdateLinks on the device (k_update_grid,
    k_update_links).  The time step is the grid's temporal spacing, as in the
    reference's Simulation (Simulation.java:394 passes tstep == at)."""

    def step(self, grid, time_step):
        grid._check_dt(time_step)
        grid.handle.update_grid()
        grid._dirty()

    def stepLinks(self, grid, time_step):
        grid._check_dt(time_step)
        grid.handle.step_links()
        grid._dirty()


class ImplicitTYMSolver(FastTYMSolver):
    """physics/fields/ImplicitTYMSolver.java: the implicit update runs on the device
    (opx_set_field_solver with OPX_SOLVER_IMPLICIT); stepLinks is FastTYMSolver's."""

    def __init__(self, implicitIterations=0, implicitDampingFactor=0.0):
        self.implicitIterations = int(implicitIterations)
        self.implicitDampingFactor = float(implicitDampingFactor)

    def clone(self):
        return ImplicitTYMSolver(self.implicitIterations, self.implicitDampingFactor)


class Grid:
    def __init__(self, settings):
        prec = N.OPX_F32 if settings.precision == "f32" else N.OPX_F64
        self.numCol = settings.numberOfColors
        if self.numCol not in (2, 3):
            raise ValueError("numberOfColors must be 2 or 3 for the Yang-Mills solver")
        if settings.numberOfDimensions != 3:
            raise ValueError("numberOfDimensions must be 3")
        self.dims = tuple(int(c) for c in settings.gridCells)
        self.a = tuple(settings.spacings)
        self.at = settings.timeStep
        self.g = settings.couplingConstant
        self.handle = N.Handle(self.numCol, self.dims, a=self.a, dt=self.at, g=self.g, precision=prec,
                               reunit_every=settings.reunitarizeEvery, device=settings.device)
        from .settings import IMPLICIT
        if settings.simulationType in IMPLICIT:
            self.fsolver = ImplicitTYMSolver(settings.implicitSolverIterations, settings.implicitSolverDamping)
            self.handle.set_field_solver(N.SOLVER_IMPLICIT, settings.implicitSolverIterations,
                                         settings.implicitSolverDamping)
        else:
            self.fsolver = FastTYMSolver()
        self.V = int(np.prod(self.dims))
        self._cache = {}
        self.simulationSteps = 0
        self.active = None
        self.evaluatable = None

    # ---- geometry (Grid.java:276-436, 736-823) ----
    def getNumCells(self, d=None):
        return list(self.dims) if d is None else self.dims[d]

    def getTotalNumberOfCells(self):
        return self.V

    def getNumberOfDimensions(self):
        return 3

    def getNumberOfColors(self):
        return self.numCol

    def getLatticeSpacing(self, i=0):
        return self.a[i]

    def getTemporalSpacing(self):
        return self.at

    def getGaugeCoupling(self):
        return self.g

    def getLatticeUnitFactor(self, i):
        return self.g * self.a[i]

    def getCellIndex(self, pos):
        p = [int(pos[i]) % self.dims[i] for i in range(3)]
        return (p[0] * self.dims[1] + p[1]) * self.dims[2] + p[2]

    def getCellPos(self, index):
        x2 = index % self.dims[2]
        t = index // self.dims[2]
        return [t // self.dims[1], t % self.dims[1], x2]

    def shift(self, index, d, o):
        p = self.getCellPos(index)
        p[d] += o
        return self.getCellIndex(p)

    # ---- regions (Grid.java:978-1004) ----
    def _region_mask(self, p1, p2):
        idx = np.indices(self.dims).reshape(3, -1)
        m = np.ones(self.V, bool)
        for j in range(3):
            m &= (idx[j] >= p1[j]) & (idx[j] <= p2[j])
        return m.astype(np.uint8)

    def setEvaluationRegion(self, p1, p2):
        self.evaluatable = self._region_mask(p1, p2)
        self.handle.set_evaluatable(self.evaluatable)

    def setActiveRegion(self, p1, p2):
        self.active = self._region_mask(p1, p2)
        self.handle.set_active(self.active)

    def isActive(self, index):
        return True if self.active is None else bool(self.active[index])

    def isEvaluatable(self, index):
        return True if self.evaluatable is None else bool(self.evaluatable[index])

    # ---- updates (Grid.java:553-593) ----
    def _check_dt(self, dt):
        if abs(dt - self.at) > 1e-15 * abs(self.at):
            raise ValueError("the device solver steps with the grid's temporal spacing")

    def updateGrid(self, tstep):
        self.fsolver.step(self, tstep)

    def updateLinks(self, tstep):
        self.fsolver.stepLinks(self, tstep)

    def storeFields(self):
        self.handle.store_fields()
        self._dirty()

    # ---- bulk field access (reference per-cell layout) ----
    def _dirty(self):
        self._cache.clear()

    def _get(self, field, layout=N.LAYOUT_REF):
        key = (field, layout)
        if key not in self._cache:
            self._cache[key] = self.handle.download(field, layout=layout)
        return self._cache[key]

    def get_links(self, t=0):
        return self._get(N.FIELD_UNEXT if t else N.FIELD_U).copy()

    def set_links(self, U, t=0):
        self.handle.upload(N.FIELD_UNEXT if t else N.FIELD_U, U)
        self._dirty()

    def get_fields(self, layout=N.LAYOUT_REF):
        return self._get(N.FIELD_E, layout).copy()

    def set_fields(self, E, layout=N.LAYOUT_REF):
        self.handle.upload(N.FIELD_E, E, layout=layout)
        self._dirty()

    def set_charge(self, rho, layout=N.LAYOUT_REF):
        self.handle.upload(N.FIELD_RHO, rho, layout=layout)
        self._dirty()

    def set_current(self, J, layout=N.LAYOUT_REF):
        self.handle.upload(N.FIELD_J, J, layout=layout)
        self._dirty()

    # ---- per-cell getters (Grid.java:126-261), read from the host mirror ----
    def getU(self, index, d):
        return self._get(N.FIELD_U)[index, d].copy()

    def getUnext(self, index, d):
        return self._get(N.FIELD_UNEXT)[index, d].copy()

    def getE(self, index, d):
        return self._get(N.FIELD_E)[index, d].copy()

    def getJ(self, index, d):
        return self._get(N.FIELD_J)[index, d].copy()

    def getRho(self, index):
        return self._get(N.FIELD_RHO)[index].copy()

    # ---- diagnostics hooks ----
    def reduce(self):
        return self.handle.reduce()

    def energy_density(self):
        return self.handle.energy_density()

    def projected_energy(self, d):
        return self.handle.projected_energy(d)

    def projected_poynting(self, d):
        """ProjectedEnergyDensity Poynting rows [2][N_d] (SU(2))."""
        return self.handle.projected_poynting(d)

    def gauss_field(self):
        return self.handle.gauss_field()

    def synchronize(self):
        self.handle.synchronize()


class Simulation:
    def __init__(self, settings):
        if settings.simulationType not in SUPPORTED:
            raise NotImplementedError(f"simulation type {settings.simulationType} is not provided by the GPU solver")
        self.settings = settings
        self.simulationType = settings.simulationType
        self.tstep = settings.timeStep
        self.iterations = settings.getIterations()
        self.totalSimulationSteps = 0
        self.totalSimulationTime = 0.0
        self.diagnostics = list(settings.diagnostics)
        self.grid = Grid(settings)
        if settings.evaluationRegionEnabled:
            self.grid.setEvaluationRegion(settings.evaluationRegionPoint1, settings.evaluationRegionPoint2)
        if settings.activeRegionEnabled:
            self.grid.setActiveRegion(settings.activeRegionPoint1, settings.activeRegionPoint2)
        self.particles = None
        for ic in settings.initialConditions:
            ic.applyInitialCondition(self)
        self.initialize()

    def getTimeStep(self):
        return self.tstep

    def getNumberOfColors(self):
        return self.settings.numberOfColors

    def getNumberOfDimensions(self):
        return 3

    def getCouplingConstant(self):
        return self.settings.couplingConstant

    def set_particles(self, pos0, pos1, vel, Q0, Q1, direction):
        """The CGC particle list (physics/particles/CGCParticle.java) as arrays."""
        self.grid.handle.particles_upload(pos0, pos1, vel, Q0, Q1, direction)
        self.particles = len(direction)

    def get_particles(self):
        """NGP particles as arrays, or the super-particle groups (optimized CGC type)."""
        if not self.particles:
            return None
        h = self.grid.handle
        from .settings import SUPER_PARTICLES
        if self.simulationType in SUPER_PARTICLES:
            return [h.super_download(k) for k in range(h.super_groups)]
        return h.particles_download()

    def initialize(self):
        """Simulation.initialize: Unext from E, then the particle phases without reassign."""
        self.grid.handle.initialize()
        self.grid._dirty()

    def step(self):
        """Simulation.step (Simulation.java:373-435): diagnostics at step 0, then one
        leapfrog update (reassign, storeFields, updateGrid, particle phases), then
        the diagnostics."""
        if self.totalSimulationSteps == 0:
            for d in self.diagnostics:
                d.initialize(self)
            self.runDiagnostics()
        self.totalSimulationSteps += 1
        self.totalSimulationTime = self.totalSimulationSteps * self.tstep
        self.grid.simulationSteps = self.totalSimulationSteps
        self.grid.handle.step(1)
        self.grid._dirty()
        self.runDiagnostics()

    def continues(self):
        return self.totalSimulationSteps <= self.iterations

    def run(self):
        """Simulation.run: step while continues().  When BulkQuantitiesInTime at
        every step is the only diagnostic, the updates after step 0 run as one
        opx_step_measured call (MainBatch's loop in one call; the same rows)."""
        if self.continues() and self._measured_loop():
            if self.totalSimulationSteps == 0:
                for d in self.diagnostics:
                    d.initialize(self)
                self.runDiagnostics()
            n = self.iterations + 1 - self.totalSimulationSteps
            rows = self.grid.handle.step_measured(n)
            self.grid._dirty()
            for o in rows:
                self.totalSimulationSteps += 1
                self.totalSimulationTime = self.totalSimulationSteps * self.tstep
                self.grid.simulationSteps = self.totalSimulationSteps
                for d in self.diagnostics:
                    d.record(o, self.totalSimulationSteps)
        while self.continues():
            self.step()

    def _measured_loop(self):
        from .diagnostics import BulkQuantitiesInTime, java_round
        if not self.diagnostics or not all(type(d) is BulkQuantitiesInTime for d in self.diagnostics):
            return False
        return all(max(java_round(d.timeInterval / self.tstep), 1) == 1 for d in self.diagnostics)

    def runDiagnostics(self):
        for d in self.diagnostics:
            d.calculate(self.grid, self.particles, self.totalSimulationSteps)
