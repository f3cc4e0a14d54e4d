"""Differentiation form, general objectives (SU(2)): the pressure anisotropy
P_L / P_T of the projected energy components (ProjectedEnergyDensity.java:18-41)
and the gradient with respect to the colour-charge density rho through Gauss's
law, checked like the energy gradient: adjoint . d against the FP64
tangent-linear run (1e-9 relative) and against central finite differences of
FP64 forward runs (h = 1e-4, 1e-5 relative).

The objective values are pinned independently: the anisotropy from the
handle's own ProjectedEnergyDensity rows after the same steps, and the charge
input against re-projecting E onto Gauss's law with the perturbed rho.
"""
import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N

pytestmark = pytest.mark.gpu


def setup(dims, seed=3, sigma=0.15):
    h = opx.Handle(2, dims, dt=0.05, precision=N.OPX_F64)
    h.init_random(seed, sigma, sigma)
    h.gauss_project(1e-26)
    return h


def unit(rng, shape):
    d = rng.normal(size=shape)
    return d / np.linalg.norm(d)


def test_anisotropy_value_matches_projected_energy(native):
    """J = sum(P_L)/sum(P_T) over a box spanning whole transverse planes equals
    the ratio formed from opx_projected_energy after the same steps."""
    dims, nsteps, l = (10, 6, 8), 7, 0
    h = setup(dims)
    lo, hi = (2, 0, 0), (6, dims[1] - 1, dims[2] - 1)
    J = h.objective_value(nsteps, N.OBJ_ANISOTROPY, l, lo, hi)
    h2 = opx.Handle(2, dims, dt=0.05)
    h2.upload(N.FIELD_U, h.download(N.FIELD_U))
    h2.upload(N.FIELD_E, h.download(N.FIELD_E))
    h2.initialize()
    h2.step(nsteps)
    rows = h2.projected_energy(l)[:, 2:7]
    t_el, t_mag, l_el, l_mag = rows.sum(axis=1)
    ref = (t_el + t_mag - l_el - l_mag) / (l_el + l_mag)
    assert abs(J - ref) <= 1e-12 * abs(ref), (J, ref)


@pytest.mark.parametrize("kind,direction", [(N.OBJ_ANISOTROPY, 0), (N.OBJ_ANISOTROPY, 2)])
def test_anisotropy_gradient_wrt_e(native, kind, direction):
    dims, nsteps = (8, 8, 8), 16
    lo, hi = (1, 2, 2), (6, 5, 6)
    h = setup(dims)
    J, g = h.objective_gradient(nsteps, 5, kind, direction, lo, hi, N.WRT_E)
    J0 = h.objective_value(nsteps, kind, direction, lo, hi)
    assert abs(J - J0) <= 1e-13 * abs(J0)
    rng = np.random.default_rng(5 + direction)
    for _ in range(4):
        d = unit(rng, g.shape)
        adj = float((g * d).sum())
        Jt, dJ = h.objective_tangent(nsteps, kind, direction, lo, hi, dE=d)
        assert abs(Jt - J0) <= 1e-13 * abs(J0)
        assert abs(adj - dJ) <= 1e-9 * abs(dJ), (adj, dJ)
        eps = 1e-4
        fd = (h.objective_value(nsteps, kind, direction, lo, hi, dE=d, h=eps) -
              h.objective_value(nsteps, kind, direction, lo, hi, dE=d, h=-eps)) / (2 * eps)
        assert abs(fd - adj) <= 1e-5 * abs(adj), (fd, adj)


@pytest.mark.parametrize("kind", [N.OBJ_ENERGY, N.OBJ_ANISOTROPY])
def test_gradient_wrt_charge_density(native, kind):
    dims, nsteps = (8, 8, 8), 12
    lo, hi = (2, 2, 2), (5, 5, 5)
    h = setup(dims, seed=7)
    J, g = h.objective_gradient(nsteps, 4, kind, 1, lo, hi, N.WRT_RHO)
    assert g.shape == (h.V, 3)
    rng = np.random.default_rng(11 + kind)
    for _ in range(4):
        d = unit(rng, g.shape)
        adj = float((g * d).sum())
        Jt, dJ = h.objective_tangent(nsteps, kind, 1, lo, hi, drho=d)
        assert abs(adj - dJ) <= 1e-9 * abs(dJ), (adj, dJ)
        eps = 1e-4
        fd = (h.objective_value(nsteps, kind, 1, lo, hi, drho=d, h=eps) -
              h.objective_value(nsteps, kind, 1, lo, hi, drho=d, h=-eps)) / (2 * eps)
        assert abs(fd - adj) <= 1e-5 * abs(adj), (fd, adj)


def test_charge_input_is_the_gauss_projection(native):
    """The charge input moves E_0 as opx_gauss_project does: J with E_0 moved
    by eps divT K^+ d equals J of the state re-projected onto div E = eps d."""
    dims, nsteps, eps = (8, 6, 8), 5, 1e-3
    h = setup(dims, seed=4)
    rng = np.random.default_rng(2)
    d = unit(rng, (h.V, 3))
    Jmoved = h.objective_value(nsteps, N.OBJ_ENERGY, 0, drho=d, h=eps)
    h2 = opx.Handle(2, dims, dt=0.05)
    h2.upload(N.FIELD_U, h.download(N.FIELD_U))
    h2.upload(N.FIELD_E, h.download(N.FIELD_E))
    h2.upload(N.FIELD_RHO, eps * d)
    it, g2 = h2.gauss_project(1e-30, 20000)
    assert g2 < 1e-26
    Jproj = h2.objective_value(nsteps, N.OBJ_ENERGY, 0)
    assert abs(Jmoved - Jproj) <= 1e-10 * abs(Jproj), (Jmoved, Jproj)


def test_objective_errors(native):
    h = setup((4, 4, 4))
    with pytest.raises(N.OpixiError) as e:
        h.objective_value(2, 7, 0)
    assert e.value.code == N.OPX_ERR_INVALID
    with pytest.raises(N.OpixiError) as e:
        h.objective_value(2, N.OBJ_ANISOTROPY, 3)
    assert e.value.code == N.OPX_ERR_INVALID
    h3 = opx.Handle(3, (4, 4, 4))
    with pytest.raises(N.OpixiError) as e:
        h3.objective_gradient(2, 1, wrt=N.WRT_RHO)
    assert e.value.code == N.OPX_ERR_UNSUPPORTED
