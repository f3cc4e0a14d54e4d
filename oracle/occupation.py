"""CPU oracle of the Coulomb gauge and the occupation numbers (SU(2)).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``; the GPU product never
imports it.

Restates (paths relative to pixi/src/main/java/org/openpixi/pixi):
* physics/gauge/CoulombGauge.java:56-194 -- the iteration: divergence of the
  gauge field A = log U (``orc_coulomb_divergence``), Poisson solve in
  momentum space with the lattice Laplacian (numpy's FFT in place of
  JTransforms 2.4.0), g = exp(-i psi), gauge transformation
  (``orc_coulomb_apply``, physics/gauge/GaugeTransformation.java:57-90);
* diagnostics/methods/OccupationNumbersInTime.java:172-297 -- occupation
  numbers and energy density from the Fourier transforms of E and of A averaged
  over U and Unext, without the optional mirrored grid and cone windows.
"""
import ctypes as C

import numpy as np

from . import OracleGrid, _p, lib


def _inverse_laplace(dims):
    """CoulombGauge.InverseLaplaceOperator (:169-193): -0.5 / (sum cos(2 pi k_i / N_i) - 3), 0 at k = 0."""
    n0, n1, n2 = dims
    k0 = np.arange(n0)[:, None, None]
    k1 = np.arange(n1)[None, :, None]
    k2 = np.arange(n2)[None, None, :]
    den = (np.cos(2 * np.pi * k0 / float(n0)) + np.cos(2 * np.pi * k1 / float(n1))
           + np.cos(2 * np.pi * k2 / float(n2)) - 3.0)
    out = np.zeros(dims)
    nz = den != 0
    out[nz] = -0.5 / den[nz]
    out[0, 0, 0] = 0.0
    return out


def coulomb_gauge(grid: OracleGrid, max_iter=100, goal=1e-18):
    """CoulombGauge.applyGaugeTransformation (:56-75) on the grid's U, Unext, E;
    returns the list of divergences (one per iteration)."""
    if grid.nc != 2:
        raise ValueError("SU(2) only")
    L = lib()
    L.orc_coulomb_divergence.restype = C.c_double
    L.orc_coulomb_divergence.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.orc_coulomb_apply.argtypes = [C.c_void_p] * 5
    V, dims = grid.V, grid.dims
    inv = _inverse_laplace(dims)
    conv = []
    div = np.empty((3, V))
    while len(conv) < max_iter:
        s = L.orc_coulomb_divergence(grid.pp, _p(grid.U), _p(div))
        psi = np.empty((3, V))
        for c in range(3):
            f = np.fft.fftn(div[c].reshape(dims).astype(complex))
            psi[c] = np.fft.ifftn(f * inv).real.reshape(-1)
        L.orc_coulomb_apply(grid.pp, _p(np.ascontiguousarray(psi)), _p(grid.U), _p(grid.Unext), _p(grid.E))
        conv.append(s)
        if s < goal:
            break
    return conv


def occupation_numbers(grid: OracleGrid, max_iter=100, goal=1e-18):
    """OccupationNumbersInTime.calculate on a copy of the grid: returns
    (n [V][3], energy density, divergence list).  Isotropic lattice spacing."""
    g = grid.copy()
    conv = coulomb_gauge(g, max_iter, goal)
    V, dims = g.V, g.dims
    a = g.a[0]
    gainv = 1.0 / (a * g.g)
    Ef = np.empty((3, 3, V))
    A = np.empty((3, 3, V))
    L = lib()
    L.orc_occupation_fields.argtypes = [C.c_void_p] * 4 + [C.c_double, C.c_void_p, C.c_void_p]
    L.orc_occupation_fields(g.pp, _p(g.U), _p(g.Unext), _p(g.E), gainv, _p(Ef), _p(A))
    eF = np.fft.fftn(Ef.reshape(3, 3, *dims), axes=(2, 3, 4)).reshape(3, 3, V)
    aF = np.fft.fftn(A.reshape(3, 3, *dims), axes=(2, 3, 4)).reshape(3, 3, V)
    deff = sum(1 for d in dims if d > 1)
    conv_f = a ** (2 * deff)
    # lattice momenta and the abelian lattice dispersion (:301-312, :334-355)
    idx = np.arange(V)
    pos = np.stack([idx // (dims[1] * dims[2]), (idx // dims[2]) % dims[1], idx % dims[2]])
    w2 = np.zeros(V)
    for i in range(3):
        delta = pos[i] / float(dims[i])
        k = np.where(delta < 0.5, 2.0 * delta * np.pi / a, 2.0 * (delta - 1.0) * np.pi / a)
        w2 += 2.0 * (1.0 - np.cos(k * a)) / (a * a)
    w = np.sqrt(w2)
    n = np.empty((V, 3))
    for k in range(3):
        e2 = sum(eF[j, k].real ** 2 + eF[j, k].imag ** 2 for j in range(3))
        a2 = sum(aF[j, k].real ** 2 + aF[j, k].imag ** 2 for j in range(3))
        mixed = -sum(2.0 * (-aF[j, k].imag * eF[j, k].real + aF[j, k].real * eF[j, k].imag) for j in range(3))
        n[:, k] = (e2 + w * w * a2 + w * mixed) * conv_f
    box = np.prod([dims[i] * g.a[i] for i in range(3) if dims[i] > 1])
    energy = n.sum() / (2.0 * box * box)
    return n, energy, conv
