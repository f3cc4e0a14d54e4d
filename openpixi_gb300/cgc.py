"""CGC initial conditions (physics/initial/CGC) on the GPU solver.

``MVModel`` holds the constructor arguments of physics/initial/CGC/MVModel.java:84-99
and ``CGCInitialCondition`` follows CGCInitialCondition.applyInitialCondition
(:55-93): charges, the improved light-cone Poisson solver
(LightConePoissonSolverImproved) and the NGP particle creator
(LightConeNGPParticleCreator), all done by ``opx_cgc_mv`` on the device; the
optional Wilson-line tadpole and dipole (WilsonLineObservables) by
``opx_cgc_wilson_lines``.
YAML: ``initialConditions: CGC: {poissonSolver, MVModel: [...]}``
(ui/util/yaml/initial/YamlCGC.java, YamlMVModel.java).
"""

class MVModel:
    """IInitialChargeDensity of the MV model with longitudinal randomness."""

    def __init__(self, direction, orientation, location, longitudinalWidth, mu, useSeed, seed,
                 ultravioletCutoffTransverse=4.44, longitudinalCoherenceLength=0.0, infraredCoefficient=0.0):
        self.direction = int(direction)
        self.orientation = int(orientation)
        self.location = float(location)
        self.longitudinalWidth = float(longitudinalWidth)
        self.mu = float(mu)
        self.useSeed = bool(useSeed)
        self.seed = int(seed)
        self.ultravioletCutoffTransverse = float(ultravioletCutoffTransverse)
        self.longitudinalCoherenceLength = float(longitudinalCoherenceLength)
        self.infraredCoefficient = float(infraredCoefficient)

    def getDirection(self):
        return self.direction

    def getOrientation(self):
        return self.orientation

    def getInfo(self):
        return "MV, mu: %f, w: %f, UVT: %f, c: %f, m: %f" % (
            self.mu, self.longitudinalWidth, self.ultravioletCutoffTransverse,
            self.longitudinalCoherenceLength, self.infraredCoefficient)

    def as_nucleus(self):
        return {"direction": self.direction, "orientation": self.orientation, "location": self.location,
                "width": self.longitudinalWidth, "mu": self.mu, "use_seed": int(self.useSeed),
                "seed": self.seed, "uvt": self.ultravioletCutoffTransverse,
                "coherence": self.longitudinalCoherenceLength, "ir": self.infraredCoefficient}


POISSON_SOLVERS = ("improved",)


class CGCInitialCondition:
    def __init__(self, chargeDensity=None, poissonSolver="improved"):
        self.initialChargeDensity = chargeDensity
        self.setPoissonSolver(poissonSolver)
        self.computeTadpole = False
        self.computeDipole = False
        self.tadpoleFilename = "tadpole.txt"
        self.dipoleFilename = "dipole.txt"

    def setInitialChargeDensity(self, rho):
        self.initialChargeDensity = rho

    def setPoissonSolver(self, name):
        # YamlCGC.getPoissonSolver: missing or unknown names fall back to "improved"
        key = (name or "improved").lower().strip()
        if key in ("regular", "improved full", "refined"):
            raise NotImplementedError(f"Poisson solver '{key}' is not provided by the GPU solver")
        self.poissonSolver = "improved"

    def applyInitialCondition(self, s):
        # the particle creator follows the simulation type (CGCInitialCondition.java:76-87)
        from .settings import SUPER_PARTICLES
        if s.simulationType not in ("TemporalCGCNGP", "TemporalImplicitCGCNGP", "TemporalOptimizedCGCNGP",
                                    "TemporalOptimizedImplicitCGCNGP"):
            raise RuntimeError("CGCInitialCondition: simulation type not supported!")
        h = s.grid.handle
        if s.simulationType in SUPER_PARTICLES:
            # LightConeNGPSuperParticleCreator: CGCSuperParticle groups
            h.cgc_mv_super([self.initialChargeDensity.as_nucleus()])
            s.particles = h.super_groups
        else:
            # LightConeNGPParticleCreator: CGCParticle list
            h.cgc_mv([self.initialChargeDensity.as_nucleus()])
            s.particles = h.np
        if self.computeTadpole or self.computeDipole:
            self._wilson_line_observables(h, s)
        s.grid._dirty()

    def _wilson_line_observables(self, h, s):
        """WilsonLineObservables.computeTadpole / computeDipole
        (physics/initial/CGC/WilsonLineObservables.java:37-131), appended to the
        files in the reference's format (FileFunctions.getFile: relative paths
        go under output/)."""
        from .diagnostics import java_sci
        tadpole, dipole, ds = h.cgc_wilson_lines(0, dipole=self.computeDipole)
        info = self.initialChargeDensity.getInfo()
        if self.computeTadpole:
            with open(_output_file(self.tadpoleFilename), "a") as f:
                f.write(info + ", V: " + java_sci(tadpole) + "\n")
        if self.computeDipole:
            with open(_output_file(self.dipoleFilename), "a") as f:
                f.write(info + "\n")
                f.write("d\ttr(V V^t)\n")
                for b, v in enumerate(dipole):
                    f.write(java_sci(b * ds) + "\t" + java_sci(v) + "\n")

    @staticmethod
    def from_yaml(cgc):
        """YamlCGC.applyTo: one CGCInitialCondition per MVModel entry."""
        others = [k for k in ("MVModelCoherent", "NucleusCoherent", "Nucleus", "NucleusThick") if cgc.get(k)]
        if others:
            raise NotImplementedError(f"CGC charge models not provided: {others}")
        out = []
        for m in cgc.get("MVModel") or []:
            seed = m.get("randomSeed")
            rho = MVModel(m["direction"], m["orientation"], m["longitudinalLocation"], m["longitudinalWidth"],
                          m["mu"], seed is not None, seed if seed is not None else 0,
                          m.get("ultravioletCutoffTransverse", 4.44), m.get("longitudinalCoherenceLength", 0.0),
                          m.get("infraredCoefficient", 0.0))
            ic = CGCInitialCondition(rho, cgc.get("poissonSolver"))
            ic.computeTadpole = bool(cgc.get("computeTadpole", False))
            ic.computeDipole = bool(cgc.get("computeDipole", False))
            ic.tadpoleFilename = cgc.get("tadpoleFilename", "tadpole.txt")
            ic.dipoleFilename = cgc.get("dipoleFilename", "dipole.txt")
            out.append(ic)
        return out


def _output_file(path):
    """FileFunctions.getFile (diagnostics/FileFunctions.java:16-32): relative
    paths are prefixed with output/, and the parent folder is created."""
    import os
    p = path if path.startswith("/") else os.path.join("output", path)
    os.makedirs(os.path.dirname(p) or ".", exist_ok=True)
    return p


__all__ = ["MVModel", "CGCInitialCondition"]
