"""Super-particle CPIC (simulationType "temporal optimized cgc ngp") on the GPU
against the oracle, through the C ABI.

From an identical state the charge density, the current and the transported
charges are bit-exact (CGCSuperParticleInterpolationNGP's sums in list order);
the initial condition agrees with the oracle to FFT rounding (1e-10), and a
coupled collision run keeps fields within 1e-10 and the Gauss law where the
initial condition put it."""
import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N
from tests.helpers import link_rel_err, field_rel_err, to_gen

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


def nuclei_args(nuclei):
    return [{"direction": 0, "orientation": n.orientation, "location": n.location, "width": n.width,
             "mu": n.mu, "use_seed": 1, "seed": n.seed, "uvt": n.uvt, "coherence": n.coherence, "ir": n.ir}
            for n in nuclei]


def collision(nc=2, dims=(40, 6, 6), dt=0.5):
    from oracle import cgc
    return [cgc.MVNucleus(orientation=1, location=12.0, width=1.5, mu=0.5, seed=3),
            cgc.MVNucleus(orientation=-1, location=28.0, width=1.5, mu=0.5, seed=4)]


@pytest.mark.parametrize("nc,dt", [(2, 0.5), (2, 0.25), (3, 0.5)])
def test_super_initial_condition_vs_oracle(native, orc, nc, dt):
    from oracle import cgc
    dims = (32, 6, 6) if nc == 3 else (40, 6, 6)
    nuclei = [cgc.MVNucleus(orientation=1, location=10.0, width=1.5, mu=0.5, seed=3),
              cgc.MVNucleus(orientation=-1, location=dims[0] - 10.0, width=1.5, mu=0.5, seed=4)]
    g = orc.OracleGrid(nc, dims, dt=dt)
    groups, _ = cgc.cgc_mv_super(g, nuclei)
    h = opx.Handle(nc, dims, dt=dt)
    h.cgc_mv_super(nuclei_args(nuclei))
    assert link_rel_err(h.download(N.FIELD_U), g.U) < 1e-10
    assert field_rel_err(h.download(N.FIELD_E), g.E) < 1e-10
    assert h.super_groups == len(groups)
    for k, G in enumerate(groups):
        d = h.super_download(k)
        assert (d["orientation"], d["n"], d["base"]) == (G.orientation, G.n, G.base)
        assert np.abs(d["Q"] - G.Q[:, :G.n]).max() <= 1e-10 * np.abs(G.Q).max()


def test_super_phases_bit_exact(native, orc):
    """Identical fields and charges: rho, J and the transported charges of
    initialize (t = 0) are bit-identical to the oracle's in the reference's
    list order for numberOfThreads = 1 (one subdivision per nucleus: every
    cell sums its terms nucleus by nucleus, k ascending).  Other thread counts
    reorder the terms at subdivision boundaries, which changes the last bit
    where two nuclei overlap."""
    from oracle import cgc
    nuclei = collision()
    g = orc.OracleGrid(2, (40, 6, 6), dt=0.5)
    groups, _ = cgc.cgc_mv_super(g, nuclei)
    g.random_links(9, 0.3)          # a non-trivial Unext for the transport
    g.Unext[...] = g.U
    h = opx.Handle(2, g.dims, dt=0.5)
    h.upload(N.FIELD_UNEXT, g.Unext)
    for G in groups:
        h.super_upload(G.orientation, G.n, G.base, G.Q[:, :G.n])
    h.cpic_phases(reassign=False)
    sim = cgc.OracleSuperSimulation(g, groups, nthreads=1)
    sim._phases(0)
    assert same_bits(h.download(N.FIELD_RHO, layout=N.LAYOUT_GEN), to_gen(orc, 2, g.rho))
    assert same_bits(h.download(N.FIELD_J, layout=N.LAYOUT_GEN), to_gen(orc, 2, g.J))
    assert np.abs(g.J).max() > 0
    for k, G in enumerate(groups):
        assert same_bits(h.super_download(k)["Q"], G.Q[:, :G.n])


@pytest.mark.parametrize("dt", [0.5, 1.0 / 3.0])
def test_super_collision_run(native, orc, dt):
    """Initialize and 3 * round(a/dt) + 1 steps: every crossing phase of every
    super particle; fields 1e-10, charges and deposits 1e-10 of their scale."""
    from oracle import cgc
    nuclei = collision()
    g = orc.OracleGrid(2, (40, 6, 6), dt=dt)
    groups, _ = cgc.cgc_mv_super(g, nuclei)
    h = opx.Handle(2, g.dims, dt=dt)
    h.upload(N.FIELD_U, g.U)
    h.upload(N.FIELD_UNEXT, g.Unext)
    h.upload(N.FIELD_E, g.E)
    for G in groups:
        h.super_upload(G.orientation, G.n, G.base, G.Q[:, :G.n])
    sim = cgc.OracleSuperSimulation(g, groups)
    sim.initialize()
    h.initialize()
    g0 = np.abs(g.gauss_field()).max()
    ppc = int(round(1.0 / dt))
    for _ in range(3 * ppc + 1):
        sim.step()
        h.step(1)
    assert link_rel_err(h.download(N.FIELD_U), g.U) <= 1e-10
    assert field_rel_err(h.download(N.FIELD_E), g.E) <= 1e-10
    rho, J = to_gen(orc, 2, g.rho), to_gen(orc, 2, g.J)
    assert np.abs(h.download(N.FIELD_RHO, layout=N.LAYOUT_GEN) - rho).max() <= 1e-10 * np.abs(rho).max()
    assert np.abs(h.download(N.FIELD_J, layout=N.LAYOUT_GEN) - J).max() <= 1e-10 * max(np.abs(J).max(), 1e-30)
    for k, G in enumerate(groups):
        assert np.abs(h.super_download(k)["Q"] - G.Q[:, :G.n]).max() <= 1e-10 * np.abs(G.Q).max()
    if ppc % 2 == 0:
        # with an even number of particles per cell the charges sit where the
        # initial Gauss violation was; odd counts leave a violation that moves
        assert np.abs(h.gauss_field()).max() <= 1.01 * g0 + 1e-12


def test_super_and_ngp_exclusive(native):
    h = opx.Handle(2, (16, 4, 4), dt=0.5)
    h.super_upload(1, 16, 0, np.zeros((2, 16, 3)))
    with pytest.raises(opx.OpixiError):
        h.particles_upload(np.zeros((1, 3)), np.zeros((1, 3)), np.zeros((1, 3)), np.zeros((1, 3)),
                           np.zeros((1, 3)), np.zeros(1, np.int32))


def test_yaml_optimized_cgc_simulation(native, tmp_path):
    """A YAML deck of the optimized CGC type through Settings / Simulation: the
    MV nuclei become super-particle groups, and the run writes the
    BulkQuantities and ProjectedEnergyDensity files (energy and Poynting rows)."""
    from openpixi_gb300 import settings as S
    from openpixi_gb300.simulation import Simulation
    bulk, proj = tmp_path / "bulk.txt", tmp_path / "proj.txt"
    deck = f"""
simulationType: temporal optimized cgc ngp
gridStep: 1
couplingConstant: 1
numberOfDimensions: 3
numberOfColors: 2
numberOfThreads: 1
gridCells: [40, 6, 6]
timeStep: 0.5
duration: 3
initialConditions:
  CGC:
    poissonSolver: improved
    MVModel:
      - direction: 0
        orientation: 1
        longitudinalLocation: 12
        longitudinalWidth: 1.5
        randomSeed: 3
        mu: 0.5
      - direction: 0
        orientation: -1
        longitudinalLocation: 28
        longitudinalWidth: 1.5
        randomSeed: 4
        mu: 0.5
output:
  bulkQuantitiesInTime:
    - path: {bulk}
      interval: 0.5
  projectedEnergyDensity:
    - path: {proj}
      interval: 1.0
      direction: 0
"""
    st = S.settings_from_string(deck)
    sim = Simulation(st)
    assert sim.simulationType == "TemporalOptimizedCGCNGP"
    assert sim.grid.handle.super_groups == 2
    sim.run()
    lines = bulk.read_text().splitlines()
    assert len(lines) >= 6
    blocks = proj.read_text().splitlines()
    assert len(blocks) % 7 == 0 and len(blocks[1].split("\t")) == 40
