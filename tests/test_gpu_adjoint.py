"""Differentiation form (SU(2)): the adjoint gradient of the box-averaged energy
density after N steps with respect to the initial E field, checked against an
FP64 tangent-linear run (dual numbers through the forward kernels) and central
finite differences (h = 1e-4) of FP64 forward runs.

Tolerances: adjoint . d against the tangent-linear dJ: 1e-9 relative when the
forward is FP64 (both are FP64 models of the same trajectory); 5e-5 when the
forward is FP32 (the FP32 trajectory itself differs from the FP64 one; about
1.3e-5 is measured on 12^3 x 30 steps).  Against central differences
(h = 1e-4): 1e-5 relative.
"""
import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N

pytestmark = pytest.mark.gpu


def setup(dims, precision=N.OPX_F64, seed=3, sigma=0.1):
    h = opx.Handle(2, dims, dt=0.05, precision=precision, reunit_every=10 if precision == N.OPX_F32 else 0)
    h.init_random(seed, sigma, sigma)
    h.gauss_project(1e-24)
    return h


@pytest.mark.parametrize("ckpt", [4, 7, 30])
def test_gradient_matches_tangent_linear_and_fd(native, ckpt):
    dims, nsteps = (8, 8, 8), 20
    lo, hi = (2, 2, 2), (5, 5, 5)
    h = setup(dims)
    J, g = h.energy_gradient(nsteps, ckpt, lo, hi)
    J0 = h.energy_objective(nsteps, lo, hi)
    assert abs(J - J0) <= 1e-13 * abs(J0)
    rng = np.random.default_rng(ckpt)
    for _ in range(6):
        d = rng.normal(size=g.shape)
        adj = float((g * d).sum())
        Jt, dJ = h.energy_tangent(nsteps, d, lo, hi)
        assert abs(Jt - J0) <= 1e-13 * abs(J0)
        assert abs(adj - dJ) <= 1e-9 * abs(dJ), (adj, dJ)
        eps = 1e-4
        fd = (h.energy_objective(nsteps, lo, hi, d, eps) - h.energy_objective(nsteps, lo, hi, d, -eps)) / (2 * eps)
        assert abs(fd - adj) <= 1e-5 * abs(adj), (fd, adj)


def test_gradient_fp32_forward(native):
    """FP32 forward with FP64 checkpoints against the FP64 tangent-linear model."""
    dims, nsteps = (12, 12, 12), 30
    h32 = setup(dims, N.OPX_F32)
    h64 = opx.Handle(2, dims, dt=0.05)
    h64.upload(N.FIELD_U, h32.download(N.FIELD_U))
    h64.upload(N.FIELD_E, h32.download(N.FIELD_E))
    lo, hi = (3, 3, 3), (8, 8, 8)
    J, g = h32.energy_gradient(nsteps, 6, lo, hi)
    rng = np.random.default_rng(9)
    for _ in range(4):
        d = rng.normal(size=g.shape)
        _, dJ = h64.energy_tangent(nsteps, d, lo, hi)
        assert abs(float((g * d).sum()) - dJ) <= 5e-5 * abs(dJ)


def test_gradient_is_local_in_time(native):
    """After N steps the gradient vanishes outside the box's causal region
    (the update couples nearest neighbours only)."""
    dims, nsteps = (16, 16, 16), 3
    h = setup(dims)
    J, g = h.energy_gradient(nsteps, 2, (7, 7, 7), (8, 8, 8))
    x = np.indices(dims).reshape(3, -1).T
    dist = np.max(np.maximum(np.maximum(0, 7 - x), np.maximum(0, x - 8)), axis=1)
    far = dist > nsteps + 2
    assert np.abs(g[far]).max() == 0.0
    assert np.abs(g[~far]).max() > 0.0


def test_su3_is_unsupported(native):
    h = opx.Handle(3, (4, 4, 4))
    with pytest.raises(N.OpixiError) as e:
        h.energy_gradient(2, 1)
    assert e.value.code == N.OPX_ERR_UNSUPPORTED


def test_differentiation_workload_64cube(native):
    """The differentiation workload: 64^3, 200 steps, dt = 0.05, checkpoints every
    14 steps, central 16^3 box, initial fields sigma = 0.1; gradient from the
    FP64 forward checked on 64 random directions against the FP64 tangent-linear
    run (1e-9) and central differences (1e-5); the FP32-forward gradient against
    the same (1e-3: over 200 steps the FP32 trajectory's own rounding grows
    chaotically to about 3e-4 relative in the gradient)."""
    dims, nsteps, ckpt = (64, 64, 64), 200, 14
    lo, hi = (24, 24, 24), (39, 39, 39)
    h64 = setup(dims, N.OPX_F64, seed=5)
    h32 = opx.Handle(2, dims, dt=0.05, precision=N.OPX_F32, reunit_every=10)
    h32.upload(N.FIELD_U, h64.download(N.FIELD_U))
    h32.upload(N.FIELD_E, h64.download(N.FIELD_E))
    J, g64 = h64.energy_gradient(nsteps, ckpt, lo, hi)
    _, g32 = h32.energy_gradient(nsteps, ckpt, lo, hi)
    rng = np.random.default_rng(64)
    worst = {"tl": 0.0, "fd": 0.0, "f32": 0.0}
    for k in range(64):
        d = rng.normal(size=g64.shape)
        adj = float((g64 * d).sum())
        _, dJ = h64.energy_tangent(nsteps, d, lo, hi)
        worst["tl"] = max(worst["tl"], abs(adj - dJ) / abs(dJ))
        worst["f32"] = max(worst["f32"], abs(float((g32 * d).sum()) - dJ) / abs(dJ))
        if k < 16:  # central differences on a subset keeps the test short; all 64 in bench
            eps = 1e-4
            fd = (h64.energy_objective(nsteps, lo, hi, d, eps) - h64.energy_objective(nsteps, lo, hi, d, -eps)) / (2 * eps)
            worst["fd"] = max(worst["fd"], abs(fd - adj) / abs(adj))
    print("differentiation workload worst relative errors:", worst)
    assert worst["tl"] <= 1e-9 and worst["fd"] <= 1e-5 and worst["f32"] <= 1e-3
