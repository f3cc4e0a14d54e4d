"""Settings and YAML input: the host-side mirror of physics/Settings.java and
ui/util/yaml/YamlSettings.java for the leapfrog / CPIC path.

Names follow the reference (camelCase accessors are kept beside snake_case
ones where the Java API is called by name from ported drivers).
"""
import math

from . import yaml_lite

# YamlSettings.applyTo simulationType map (ui/util/yaml/YamlSettings.java:59-74)
SIMULATION_TYPES = {
    "temporal yang-mills": "TemporalYangMills",
    "temporal cgc": "TemporalCGC",
    "temporal cgc ngp": "TemporalCGCNGP",
    "temporal implicit cgc ngp": "TemporalImplicitCGCNGP",
    "temporal optimized cgc ngp": "TemporalOptimizedCGCNGP",
    "temporal optimized implicit cgc ngp": "TemporalOptimizedImplicitCGCNGP",
    "boost-invariant cgc": "BoostInvariantCGC",
}
# simulation types whose solver/interpolator combination this library provides
# (Settings.applySimulationTypeSetting, physics/Settings.java:540-581)
SUPPORTED = {"TemporalYangMills", "TemporalCGCNGP", "TemporalOptimizedCGCNGP", "TemporalImplicitCGCNGP",
             "TemporalOptimizedImplicitCGCNGP"}
IMPLICIT = {"TemporalImplicitCGCNGP", "TemporalOptimizedImplicitCGCNGP"}
SUPER_PARTICLES = {"TemporalOptimizedCGCNGP", "TemporalOptimizedImplicitCGCNGP"}


class Settings:
    """physics/Settings.java defaults (:43-104)."""

    def __init__(self):
        self.simulationType = "TemporalYangMills"
        self.numberOfColors = 2
        self.numberOfDimensions = 3
        self.couplingConstant = 1.0
        self.timeStep = 0.1
        self.gridStep = 1.0
        self.gridSteps = None
        self.tMax = 1000.0
        self.gridCells = [1, 1, 1]
        self.numOfThreads = 1
        self.speedOfLight = 1.0
        self.evaluationRegionEnabled = False
        self.evaluationRegionPoint1 = None
        self.evaluationRegionPoint2 = None
        self.activeRegionEnabled = False
        self.activeRegionPoint1 = None
        self.activeRegionPoint2 = None
        self.diagnostics = []
        self.initialConditions = []
        self.particles = []
        # device section (no counterpart in the reference)
        self.precision = "f64"
        self.reunitarizeEvery = 0
        self.device = 0
        # ImplicitTYMSolver parameters (Settings.java:79-80)
        self.implicitSolverIterations = 0
        self.implicitSolverDamping = 0.0

    # ---- accessors named as in Settings.java ----
    def setSimulationType(self, t):
        if t not in SIMULATION_TYPES.values():
            raise ValueError(f"unknown simulation type {t!r}")
        self.simulationType = t

    def setTimeStep(self, dt):
        self.timeStep = float(dt)

    def setTMax(self, t):
        self.tMax = float(t)

    def getIterations(self):
        # iterations = (int) Math.ceil(tMax / timeStep) (Settings.java:98, :372-380)
        return int(math.ceil(self.tMax / self.timeStep))

    def setGridStep(self, *args):
        if len(args) == 1:
            self.gridStep = float(args[0])
            self.gridSteps = None
        else:
            i, v = args
            if self.gridSteps is None:
                self.gridSteps = [self.gridStep] * self.numberOfDimensions
            self.gridSteps[i] = float(v)

    def getGridStep(self, i=None):
        if i is None:
            return self.gridStep
        return self.gridSteps[i] if self.gridSteps is not None else self.gridStep

    def setGridCells(self, i, n):
        self.gridCells[i] = int(n)

    def getGridCells(self, i):
        return self.gridCells[i]

    def setNumberOfColors(self, n):
        self.numberOfColors = int(n)

    def setNumberOfDimensions(self, n):
        self.numberOfDimensions = int(n)
        self.gridCells = [1] * self.numberOfDimensions

    def setCouplingConstant(self, g):
        self.couplingConstant = float(g)

    def setNumOfThreads(self, n):
        self.numOfThreads = int(n)

    def addDiagnostics(self, d):
        self.diagnostics.append(d)

    def addInitialConditions(self, ic):
        self.initialConditions.append(ic)

    @property
    def spacings(self):
        return [self.getGridStep(i) for i in range(3)]


def _region(d, cells):
    """YamlRegion.getPoint1/getPoint2: negative coordinates count from the end
    (ui/util/yaml/YamlRegion.java)."""
    p1 = [int(v) + (cells[i] if int(v) < 0 else 0) for i, v in enumerate(d["point1"])]
    p2 = [int(v) + (cells[i] if int(v) < 0 else 0) for i, v in enumerate(d["point2"])]
    return p1, p2


def apply_yaml(doc, settings=None):
    """YamlSettings.applyTo (ui/util/yaml/YamlSettings.java:46-191) for the keys of
    this path.  ``doc`` is the parsed YAML mapping."""
    from . import diagnostics, initial
    s = settings or Settings()
    # YAML-level defaults (YamlSettings.java:49-56)
    s.simulationType = "TemporalYangMills"
    s.speedOfLight = 1.0
    s.setNumberOfDimensions(3)
    s.setNumberOfColors(1)
    s.setCouplingConstant(1.0)
    s.setNumOfThreads(4)
    st = doc.get("simulationType")
    if st is not None:
        if st not in SIMULATION_TYPES:
            raise ValueError("Unknown simulation type specified in YAML file.")
        s.setSimulationType(SIMULATION_TYPES[st])
    if doc.get("timeStep") is not None:
        s.setTimeStep(doc["timeStep"])
    if doc.get("duration") is not None:
        s.setTMax(doc["duration"])
    if doc.get("numberOfDimensions") is not None:
        s.setNumberOfDimensions(doc["numberOfDimensions"])
    if doc.get("speedOfLight") is not None:
        s.speedOfLight = float(doc["speedOfLight"])
    if doc.get("numberOfColors") is not None:
        s.setNumberOfColors(doc["numberOfColors"])
    if doc.get("couplingConstant") is not None:
        s.setCouplingConstant(doc["couplingConstant"])
    if doc.get("numberOfThreads") is not None:
        s.setNumOfThreads(doc["numberOfThreads"])
    # YamlSettings.java:29-30, 100-105
    if doc.get("implicitSolverIterations") is not None:
        s.implicitSolverIterations = int(doc["implicitSolverIterations"])
    if doc.get("implicitSolverDamping") is not None:
        s.implicitSolverDamping = float(doc["implicitSolverDamping"])
    nd = s.numberOfDimensions
    if doc.get("gridSteps") is not None:
        if len(doc["gridSteps"]) != nd:
            raise ValueError("Size of gridSteps does not match numberOfDimensions.")
        for i, v in enumerate(doc["gridSteps"]):
            s.setGridStep(i, v)
    elif doc.get("gridStep") is not None:
        s.setGridStep(doc["gridStep"])
    cells = doc.get("gridCells")
    if cells is not None:
        if len(cells) != nd:
            raise ValueError("Size of gridCells does not match numberOfDimensions.")
        for i, v in enumerate(cells):
            s.setGridCells(i, v)
    for key, attr in (("evaluationRegion", "evaluationRegion"), ("activeRegion", "activeRegion")):
        reg = doc.get(key)
        if reg is not None and reg.get("point1") is not None and reg.get("point2") is not None \
                and len(reg["point1"]) == nd and len(reg["point2"]) == nd:
            if reg.get("enabled") is not None:
                setattr(s, attr + "Enabled", bool(reg["enabled"]))
            p1, p2 = _region(reg, s.gridCells)
            setattr(s, attr + "Point1", p1)
            setattr(s, attr + "Point2", p2)
    ics = doc.get("initialConditions")
    if ics:
        for ic in initial.from_yaml(ics):
            s.addInitialConditions(ic)
    out = doc.get("output")
    if out:
        for d in diagnostics.from_yaml(out):
            s.addDiagnostics(d)
    gpu = doc.get("gpu")
    if gpu:
        s.precision = str(gpu.get("precision", s.precision))
        s.reunitarizeEvery = int(gpu.get("reunitarizeEvery", s.reunitarizeEvery))
        s.device = int(gpu.get("device", s.device))
    return s


def settings_from_string(text):
    """YamlParser.parseString + YamlSettings.applyTo (ui/util/yaml/YamlParser.java:15-19)."""
    return apply_yaml(yaml_lite.loads(text))


def settings_from_file(path):
    return apply_yaml(yaml_lite.load(path))
