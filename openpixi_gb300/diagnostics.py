"""Diagnostics: host-side mirror of diagnostics/Diagnostics.java and the methods
of this path.  The numbers come from the device reductions (opx_reduce,
opx_energy_density, opx_projected_energy); these classes only schedule them and
write the reference's file formats.

  BulkQuantitiesInTime   diagnostics/methods/BulkQuantitiesInTime.java (TSV, :66, :83-121)
  EnergyDensity          diagnostics/methods/EnergyDensity.java (big-endian binary, :15-31, :119-166)
  ProjectedEnergyDensity diagnostics/methods/ProjectedEnergyDensity.java (TSV rows, :91-105, :114-179)
"""
import decimal
import math
import os
import struct
import time

import numpy as np

def java_round(x):
    """Math.round(double): the nearest integer, halves rounded up (the Java 7+
    definition, in which 0.49999999999999994 rounds to 0)."""
    x = float(x)
    r = math.floor(x)
    return int(r) + (1 if x - r >= 0.5 else 0)


def java_sci(x):
    """java.text.DecimalFormat("0.################E0").format(x): one integer
    digit, up to 16 fraction digits, no '+' in the exponent.  DecimalFormat
    starts from the digits of Double.toString (DigitList.set(double) takes
    FloatingDecimal's shortest round-trip digits) and rounds them (HALF_EVEN)
    only beyond the pattern's 17 significant digits, which the shortest digits
    of a double never exceed: the mantissa is the shortest round-trip digits
    (the digits of JDK 19+ Double.toString; older JDKs print one digit more
    for a few rare values)."""
    x = float(x)
    if x != x:
        return "NaN"
    if x in (float("inf"), float("-inf")):
        return ("-" if x < 0 else "") + "\u221e"
    if x == 0.0:
        return ("-" if math.copysign(1.0, x) < 0 else "") + "0E0"
    sign, digits, exp = decimal.Decimal(repr(x)).as_tuple()
    ds = "".join(str(v) for v in digits)
    lead = len(ds) - len(ds.lstrip("0"))
    ds = ds.lstrip("0")
    e10 = exp + len(digits) - lead - 1
    ds = ds.rstrip("0") or "0"
    mant = ds[0] + ("." + ds[1:] if len(ds) > 1 else "")
    return ("-" if sign else "") + mant + "E" + str(e10)


def java_double(x):
    """Double.toString(x): the shortest digits that round-trip, plain decimal
    for 1e-3 <= |x| < 1e7 (at least one fraction digit), otherwise
    d.dddE<exp> with at least one fraction digit."""
    x = float(x)
    if x != x:
        return "NaN"
    if x in (float("inf"), float("-inf")):
        return "-Infinity" if x < 0 else "Infinity"
    if x == 0.0:
        return "-0.0" if str(x).startswith("-") else "0.0"
    sign, digits, exp = decimal.Decimal(repr(x)).as_tuple()
    ds = "".join(str(v) for v in digits).lstrip("0") or "0"
    # value = 0.ds * 10^(point), point = number of digits before the decimal point
    point = len(digits) + exp - (len(digits) - len("".join(str(v) for v in digits).lstrip("0")))
    ds = ds.rstrip("0") or "0"
    neg = "-" if sign else ""
    ax = abs(x)
    if 1e-3 <= ax < 1e7:
        if point <= 0:
            return neg + "0." + "0" * (-point) + ds
        if point >= len(ds):
            return neg + ds + "0" * (point - len(ds)) + ".0"
        return neg + ds[:point] + "." + ds[point:]
    frac = ds[1:] or "0"
    return neg + ds[0] + "." + frac + "E" + str(point - 1)


class Diagnostics:
    """diagnostics/Diagnostics.java:32-51"""

    def initialize(self, simulation):
        raise NotImplementedError

    def calculate(self, grid, particles, steps):
        raise NotImplementedError


class BulkQuantitiesInTime(Diagnostics):
    HEADER = "#time \t E^2 \t B^2 \t P_x \t P_y \t P_z \t G \t rho^2"

    def __init__(self, path, time_interval, supress_output=False):
        self.path = path
        self.timeInterval = float(time_interval)
        self.supressOutput = supress_output
        self.rows = []

    def initialize(self, s):
        self.s = s
        self.stepInterval = max(java_round(self.timeInterval / s.getTimeStep()), 1)
        if not self.supressOutput:
            with open(self.path, "w") as f:
                f.write(self.HEADER + "\n")

    def calculate(self, grid, particles, steps):
        if steps % self.stepInterval != 0:
            return
        self.record(grid.reduce(), steps)

    def record(self, o, steps):
        """One row from the observables o (opx_observables) at step `steps`."""
        self.eSquared, self.bSquared = o.e2_total, o.b2_total
        self.px, self.py, self.pz = o.px, o.py, o.pz
        self.gaussViolation, self.totalChargeSquared = o.gauss, o.rho2
        row = [steps * self.s.getTimeStep(), o.e2_total, o.b2_total, o.px, o.py, o.pz, o.gauss, o.rho2]
        self.rows.append(row)
        if not self.supressOutput:
            with open(self.path, "a") as f:
                f.write("\t".join(java_sci(v) for v in row) + "\n")


class EnergyDensity(Diagnostics):
    """Per-cell energy density, one big-endian binary file per output time:
    int32 D, int32 N[D], then V float64 (Java DataOutputStream)."""

    def __init__(self, filename, start_time, time_interval):
        self.filename = filename
        self.startTime = float(start_time)
        self.timeInterval = float(time_interval)
        self.counter = 0
        self.last = None

    def file_for(self, counter):
        """FilenameUtils.concat(getPath(f), getBaseName(f) + "_" + counter + "." + getExtension(f))
        (EnergyDensity.java:62-67): the dot stays when the name has no extension."""
        head, name = os.path.split(self.filename)
        dot = name.rfind(".")
        base, ext = (name[:dot], name[dot + 1:]) if dot >= 0 else (name, "")
        return os.path.join(head, f"{base}_{counter}.{ext}")

    def initialize(self, s):
        self.firstStep = max(java_round(self.startTime / s.getTimeStep()), 1)
        self.step = java_round(self.timeInterval / s.getTimeStep())
        self.s = s

    def calculate(self, grid, particles, steps):
        if steps % self.step != 0 or steps < self.firstStep:
            return
        self.counter += 1
        path = self.file_for(self.counter)
        e = grid.energy_density()
        self.last = e
        with open(path, "wb") as f:
            f.write(struct.pack(">i", 3))
            f.write(struct.pack(">3i", *grid.dims))
            f.write(e.astype(">f8").tobytes())


class ProjectedEnergyDensity(Diagnostics):
    def __init__(self, path, time_interval, direction, compute_energy_density=True,
                 compute_poynting_vector=False):
        self.path = path
        self.timeInterval = float(time_interval)
        self.direction = int(direction)
        self.computeEnergyDensity = compute_energy_density
        self.computePoyntingVector = compute_poynting_vector
        self.last = None
        self.last_poynting = None

    def initialize(self, s):
        self.stepInterval = max(java_round(self.timeInterval / s.getTimeStep()), 1)
        open(self.path, "w").close()

    def calculate(self, grid, particles, steps):
        if steps % self.stepInterval != 0:
            return
        rows = grid.projected_energy(self.direction) if self.computeEnergyDensity else None
        prow = grid.projected_poynting(self.direction) if self.computePoyntingVector else None
        self.last = rows
        self.last_poynting = prow
        with open(self.path, "a") as f:
            f.write(java_double(steps * grid.getTemporalSpacing()) + "\n")
            for block in (rows, prow):
                if block is not None:
                    for r in block:
                        f.write("\t".join(java_sci(v) for v in r) + "\n")


class OccupationNumbersInTime(Diagnostics):
    """diagnostics/methods/OccupationNumbersInTime.java: occupation numbers in
    Coulomb gauge (SU(2), SU(3)).  CSV output: a header with the grid size
    (+ the momentum vectors for "csv_with_vectors"), then per measurement
    "time, energy" and the occupation numbers (one line per colour when
    colorful, else their colour sum); "csv_only_energy" writes the first line
    only, "none" nothing.  The options of the long constructor (:99-115): the
    Coulomb gauge on the grid mirrored along mirroredDirection, and the
    Gaussian, Tukey and rectangular (cone) windows."""

    TYPES = ("csv", "csv_only_energy", "csv_with_vectors", "none")

    def __init__(self, interval, output_type, path, colorful=False, max_iter=100, accuracy_goal=1e-18,
                 useMirroredGrid=False, mirroredDirection=0, useCone=False, collisionTime=0.0,
                 collisionPosition=(0.0, 0.0, 0.0), coneVelocity=(0.0, 0.0, 0.0), useGaussianWindow=False,
                 useTukeyWindow=False, tukeyWidth=0.0):
        self.timeInterval = float(interval)
        self.outputType = output_type
        self.path = path
        self.colorful = bool(colorful)
        self.maxIter = int(max_iter)
        self.accuracyGoal = float(accuracy_goal)
        from ._native import WINDOW_CONE, WINDOW_GAUSSIAN, WINDOW_TUKEY
        self.mirroredDirection = int(mirroredDirection) if useMirroredGrid else -1
        self.windows = ((WINDOW_GAUSSIAN if useGaussianWindow else 0) | (WINDOW_TUKEY if useTukeyWindow else 0)
                        | (WINDOW_CONE if useCone else 0))
        self.collisionTime = float(collisionTime)
        self.collisionPosition = tuple(float(v) for v in collisionPosition)
        self.coneVelocity = tuple(float(v) for v in coneVelocity)
        self.tukeyWidth = float(tukeyWidth)
        self.computationCounter = 0
        self.occupationNumbers = None
        self.energyDensity = None
        if output_type not in self.TYPES:
            raise ValueError(f"OccupationNumbersInTime: unsupported output type {output_type}")
        if output_type != "none":
            open(path, "w").close()

    def initialize(self, s):
        self.stepInterval = max(java_round(self.timeInterval / s.getTimeStep()), 1)
        dims = s.grid.dims
        if self.outputType == "none":
            return
        with open(self.path, "a") as f:
            f.write(", ".join(str(int(d)) for d in dims) + "\n")
            if self.outputType == "csv_with_vectors":
                a = s.grid.getLatticeSpacing(0)
                ks = []
                for i in range(int(np.prod(dims))):
                    pos = (i // (dims[1] * dims[2]), (i // dims[2]) % dims[1], i % dims[2])
                    k = []
                    for j in range(3):
                        delta = pos[j] / float(dims[j])
                        k.append(2.0 * delta * np.pi / a if delta < 0.5 else 2.0 * (delta - 1.0) * np.pi / a)
                    ks.append(", ".join(java_double(v) for v in k))
                f.write(", ".join(ks) + "\n")

    def calculate(self, grid, particles, steps):
        if steps % self.stepInterval != 0:
            return
        n, e, it, dv = grid.handle.occupation_numbers(self.maxIter, self.accuracyGoal,
                                                      with_n=self.outputType != "csv_only_energy",
                                                      mirrored_direction=self.mirroredDirection,
                                                      windows=self.windows, collision_time=self.collisionTime,
                                                      collision_position=self.collisionPosition,
                                                      cone_velocity=self.coneVelocity,
                                                      tukey_width=self.tukeyWidth)
        self.occupationNumbers, self.energyDensity = n, e
        if self.outputType != "none":
            with open(self.path, "a") as f:
                f.write(java_double(self.computationCounter * self.timeInterval) + ", " + java_double(e) + "\n")
                if self.outputType in ("csv", "csv_with_vectors"):
                    if self.colorful:
                        for k in range(n.shape[1]):
                            f.write(", ".join(java_double(v) for v in n[:, k]) + "\n")
                    else:
                        f.write(", ".join(java_double(v) for v in n.sum(axis=1)) + "\n")
        self.computationCounter += 1


class TimeMeasurement(Diagnostics):
    """diagnostics/methods/TimeMeasurement.java: wall time per output interval."""

    def __init__(self, path, interval):
        self.path = path
        self.interval = float(interval)

    def initialize(self, s):
        self.stepInterval = max(java_round(self.interval / s.getTimeStep()), 1)
        self.t0 = time.perf_counter()
        open(self.path, "w").close()

    def calculate(self, grid, particles, steps):
        if steps % self.stepInterval != 0:
            return
        grid.synchronize()
        with open(self.path, "a") as f:
            f.write(f"{steps}\t{time.perf_counter() - self.t0:.6f}\n")


def from_yaml(out):
    """YamlOutput.applyTo (ui/util/yaml/YamlOutput.java) for the outputs of this path."""
    ds = []
    for o in out.get("bulkQuantitiesInTime") or []:
        ds.append(BulkQuantitiesInTime(o["path"], o["interval"]))
    for o in out.get("energyDensity") or []:
        ds.append(EnergyDensity(o["path"], o.get("startTime", 0.0), o["timeInterval"]))
    for o in out.get("projectedEnergyDensity") or []:
        ds.append(ProjectedEnergyDensity(o["path"], o["interval"], o.get("direction", 0),
                                         o.get("computeEnergyDensity", True),
                                         o.get("computePoyntingVector", True)))
    for o in out.get("timeMeasurement") or []:
        ds.append(TimeMeasurement(o["path"], o["interval"]))
    for o in out.get("occupationNumbersInTime") or []:
        kw = {}
        if o.get("useMirroredGrid") is not None:
            # YamlOccupationNumbersInTime.getFileGenerator: the long constructor
            kw = dict(useMirroredGrid=bool(o["useMirroredGrid"]), mirroredDirection=o.get("mirroredDirection", 0),
                      useCone=bool(o.get("useRectangularWindow", False)),
                      collisionTime=o.get("collisionTime", 0.0),
                      collisionPosition=o.get("collisionPosition", [0.0, 0.0, 0.0]),
                      coneVelocity=o.get("coneVelocity", [0.0, 0.0, 0.0]),
                      useGaussianWindow=bool(o.get("useGaussianWindow", False)),
                      useTukeyWindow=bool(o.get("useTukeyWindow", False)), tukeyWidth=o.get("tukeyWidth", 0.0))
        ds.append(OccupationNumbersInTime(o["interval"], o["outputType"], o["path"], bool(o.get("colorful", False)),
                                          **kw))
    unsupported = set(out) - {"bulkQuantitiesInTime", "energyDensity", "projectedEnergyDensity", "timeMeasurement",
                              "occupationNumbersInTime"}
    if unsupported:
        raise NotImplementedError(f"output generators not provided: {sorted(unsupported)}")
    return ds
