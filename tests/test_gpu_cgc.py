"""CGC (MV-model) initial conditions on the GPU against the oracle, through the C ABI.

The device path (cuFFT, Wilson-line scan, improved links, particle creator and
refinement) and the oracle (numpy FFT, sequential C) share the java.util.Random
stream, so the charges agree exactly before the FFTs; afterwards fields agree
to FFT rounding (bar 1e-10), particle positions, velocities and count are
bit-exact, and particle charges agree to 1e-10 of the largest charge.  A
coupled CPIC run from these initial conditions keeps fields within 1e-10 and
the Gauss law at the level the initial condition leaves it.
"""
import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N
from tests.helpers import link_rel_err, field_rel_err

pytestmark = pytest.mark.gpu


def nuclei_args(nuclei):
    return [{"direction": 0, "orientation": n.orientation, "location": n.location, "width": n.width,
             "mu": n.mu, "use_seed": 1, "seed": n.seed, "uvt": n.uvt, "coherence": n.coherence, "ir": n.ir}
            for n in nuclei]


def run_both(nc, dims, nuclei, dt=0.5):
    import oracle
    from oracle import cgc
    g = oracle.OracleGrid(nc, dims, dt=dt)
    P, _ = cgc.cgc_mv(g, nuclei)
    h = opx.Handle(nc, dims, dt=dt)
    h.cgc_mv(nuclei_args(nuclei))
    return g, P, h


def same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


CASES = {
    "su2_two_nuclei": (2, (32, 8, 8), [dict(orientation=1, location=8.0, width=1.5, mu=0.5, seed=1),
                                       dict(orientation=-1, location=24.0, width=1.5, mu=0.5, seed=2)]),
    "su2_uv_ir_coherence": (2, (24, 12, 10), [dict(orientation=-1, location=12.0, width=2.0, mu=0.7, seed=-7,
                                                   uvt=2.0, coherence=0.5, ir=0.3)]),
    "su3_one_nucleus": (3, (24, 8, 8), [dict(orientation=1, location=12.0, width=1.5, mu=0.5, seed=5)]),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_cgc_initial_condition_vs_oracle(native, orc, case):
    from oracle import cgc
    nc, dims, spec = CASES[case]
    nuclei = [cgc.MVNucleus(**s) for s in spec]
    g, P, h = run_both(nc, dims, nuclei)
    assert link_rel_err(h.download(N.FIELD_U), g.U) < 1e-10
    assert link_rel_err(h.download(N.FIELD_UNEXT), g.Unext) < 1e-10
    assert field_rel_err(h.download(N.FIELD_E), g.E) < 1e-10
    assert np.abs(g.E).max() > 1e-3
    assert h.np == P.n and P.n > 0
    d = h.particles_download()
    for k in ("pos0", "pos1", "vel"):
        assert same_bits(d[k], getattr(P, k)), k
    assert np.array_equal(d["dir"], P.dir)
    qmax = np.abs(P.Q0).max()
    assert np.abs(d["Q0"] - P.Q0).max() <= 1e-10 * qmax
    assert same_bits(d["Q0"], d["Q1"])


def test_cgc_appends_to_existing_particles(native, orc):
    """Applying the nuclei one call at a time (one CGCInitialCondition per YAML
    entry) gives the same state and particle list as one call with both."""
    from oracle import cgc
    nc, dims, spec = CASES["su2_two_nuclei"]
    nuclei = [cgc.MVNucleus(**s) for s in spec]
    h1 = opx.Handle(nc, dims, dt=0.5)
    h1.cgc_mv(nuclei_args(nuclei))
    h2 = opx.Handle(nc, dims, dt=0.5)
    for nu in nuclei_args(nuclei):
        h2.cgc_mv([nu])
    assert h1.np == h2.np
    a, b = h1.particles_download(), h2.particles_download()
    for k in ("pos0", "pos1", "vel", "Q0", "Q1", "dir"):
        assert same_bits(a[k], b[k]), k
    assert same_bits(h1.download(N.FIELD_U), h2.download(N.FIELD_U))


def test_cgc_collision_run_vs_oracle(native, orc):
    """Two nuclei, Simulation.initialize and 40 CPIC steps (temporal cgc ngp)."""
    from oracle import cgc
    nc, dims = 2, (40, 8, 8)
    nuclei = [cgc.MVNucleus(orientation=1, location=12.0, width=1.5, mu=0.5, seed=3),
              cgc.MVNucleus(orientation=-1, location=28.0, width=1.5, mu=0.5, seed=4)]
    g, P, h = run_both(nc, dims, nuclei)
    sim = orc.OracleSimulation(g, P)
    sim.initialize()
    h.initialize()
    g0 = np.abs(g.gauss_field()).max()
    for _ in range(40):
        sim.step()
    h.step(40)
    assert link_rel_err(h.download(N.FIELD_U), g.U) < 1e-10
    assert field_rel_err(h.download(N.FIELD_E), g.E) < 1e-10
    d = h.particles_download()
    assert same_bits(d["pos0"], P.pos0)
    qmax = np.abs(P.Q0).max()
    assert np.abs(d["Q0"] - P.Q0).max() <= 1e-9 * qmax
    bo, bd = g.bulk(), h.reduce()
    assert abs(bd.e2_total - bo[11]) <= 1e-10 * bo[11] and abs(bd.b2_total - bo[12]) <= 1e-10 * bo[12]
    # the Gauss law holds through the run as well as the initial condition set it up
    assert np.abs(g.gauss_field()).max() <= 1.01 * g0 + 1e-12
    assert np.abs(h.gauss_field()).max() <= 1.01 * g0 + 1e-12


def test_cgc_rejects_bad_input(native):
    h = opx.Handle(2, (16, 8, 8), dt=0.5)
    nu = nuclei_args([type("Nu", (), dict(orientation=2, location=8.0, width=1.0, mu=0.5, seed=1, uvt=4.44,
                                          coherence=0.0, ir=0.0))])
    with pytest.raises(opx.OpixiError):
        h.cgc_mv(nu)
    nu[0]["orientation"], nu[0]["direction"] = 1, 1
    with pytest.raises(opx.OpixiError):
        h.cgc_mv(nu)
    hf = opx.Handle(2, (16, 8, 8), dt=0.5, precision=N.OPX_F32)
    nu[0]["direction"] = 0
    with pytest.raises(opx.OpixiError):
        hf.cgc_mv(nu)


@pytest.mark.parametrize("case", ["su2_two_nuclei", "su3_one_nucleus", "su2_uv_ir_coherence"])
def test_wilson_line_observables_vs_oracle(native, orc, case):
    """WilsonLineObservables (tadpole, binned dipole) of every nucleus from the
    device's Wilson lines against the oracle's (FFT rounding: 1e-10)."""
    import oracle
    from oracle import cgc
    nc, dims, spec = CASES[case]
    nuclei = [cgc.MVNucleus(**s) for s in spec]
    g = oracle.OracleGrid(nc, dims, dt=0.5)
    _, info = cgc.cgc_mv(g, nuclei)
    h = opx.Handle(nc, dims, dt=0.5)
    h.cgc_mv(nuclei_args(nuclei))
    for k, d in enumerate(info):
        t_ref = cgc.wilson_tadpole(d["vt"], nc)
        dip_ref, ds_ref = cgc.wilson_dipole(d["vt"], nc, dims[1], dims[2])
        t, dip, ds = h.cgc_wilson_lines(k)
        assert abs(t - t_ref) <= 1e-10 * nc, (k, t, t_ref)
        assert ds == ds_ref
        assert np.allclose(dip, dip_ref, rtol=0, atol=1e-10 * nc, equal_nan=True), (dip, dip_ref)
        assert abs(t) < nc  # the nucleus rotates the Wilson lines away from the identity
    with pytest.raises(opx.OpixiError):
        h.cgc_wilson_lines(len(info))


def test_wilson_line_files(native, tmp_path, monkeypatch):
    """CGCInitialCondition with computeTadpole / computeDipole writes the
    reference's files under output/: '<info>, V: <mean>' and the dipole table."""
    from openpixi_gb300.cgc import CGCInitialCondition, MVModel
    from openpixi_gb300.settings import Settings
    from openpixi_gb300.simulation import Simulation
    monkeypatch.chdir(tmp_path)
    st = Settings()
    for i, n in enumerate((24, 8, 8)):
        st.setGridCells(i, n)
    st.setGridStep(1.0)
    st.setTimeStep(0.5)
    st.setCouplingConstant(1.0)
    st.setSimulationType("TemporalCGCNGP")
    ic = CGCInitialCondition(MVModel(0, 1, 12.0, 1.5, 0.5, True, 3))
    ic.computeTadpole = ic.computeDipole = True
    st.addInitialConditions(ic)
    Simulation(st)
    lines = (tmp_path / "output" / "tadpole.txt").read_text().splitlines()
    assert len(lines) == 1 and lines[0].startswith("MV, mu: 0.500000, w: 1.500000, UVT: 4.440000") and ", V: " in lines[0]
    dip = (tmp_path / "output" / "dipole.txt").read_text().splitlines()
    assert dip[1] == "d\ttr(V V^t)" and len(dip) == 2 + 4
