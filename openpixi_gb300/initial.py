"""Initial conditions (physics/initial/IInitialCondition.java): applied by the
Simulation constructor before initialize() (Simulation.java:274-276).

  RandomGaussianFields  seeded synthetic fields for the pure Yang-Mills
                        workloads: U_i(x) = exp(i A_i^a(x) t_a), A ~ N(0, sigmaA^2),
                        E_i^a(x) ~ N(0, sigmaE^2) projected onto Gauss's law
                        (no counterpart in the reference, whose random field
                        generator SU2RandomFields is unseeded)
  CGCInitialCondition   physics/initial/CGC/CGCInitialCondition.java (MV model
                        nuclei, FFT Poisson solve, Wilson lines)
"""


class IInitialCondition:
    def applyInitialCondition(self, simulation):
        raise NotImplementedError


class RandomGaussianFields(IInitialCondition):
    def __init__(self, seed, sigma_a, sigma_e, gauss_project=True, tol=1e-26, maxit=5000):
        self.seed = int(seed)
        self.sigmaA = float(sigma_a)
        self.sigmaE = float(sigma_e)
        self.gaussProject = bool(gauss_project)
        self.tol = float(tol)
        self.maxit = int(maxit)
        self.cg_iterations = None
        self.final_g2 = None

    def applyInitialCondition(self, s):
        h = s.grid.handle
        h.init_random(self.seed, self.sigmaA, self.sigmaE)
        if self.gaussProject:
            self.cg_iterations, self.final_g2 = h.gauss_project(self.tol, self.maxit)
        s.grid._dirty()


def from_yaml(ics):
    """initialConditions section (ui/util/yaml/YamlInitialConditions.java) for this path."""
    out = []
    for o in ics.get("randomGaussian") or []:
        out.append(RandomGaussianFields(o.get("randomSeed", 0), o.get("sigmaA", 0.1), o.get("sigmaE", 0.1),
                                        o.get("gaussProject", True)))
    if ics.get("CGC") is not None:
        from .cgc import CGCInitialCondition
        out.extend(CGCInitialCondition.from_yaml(ics["CGC"]))
    unsupported = set(ics) - {"randomGaussian", "CGC"}
    if unsupported:
        raise NotImplementedError(f"initial conditions not provided: {sorted(unsupported)}")
    return out
