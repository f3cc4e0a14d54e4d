"""CPU oracle of the Coulomb gauge and the occupation numbers (SU(2), SU(3)).

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
    L = lib()
    L.orc_coulomb_divergence.restype = C.c_double
    L.orc_coulomb_divergence.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.orc_coulomb_apply.argtypes = [C.c_void_p] * 5
    V, dims = grid.V, grid.dims
    ncomp = 3 if grid.nc == 2 else 8
    inv = _inverse_laplace(dims)
    conv = []
    div = np.empty((ncomp, V))
    while len(conv) < max_iter:
        s = L.orc_coulomb_divergence(grid.pp, _p(grid.U), _p(div))
        psi = np.empty((ncomp, V))
        for c in range(ncomp):
            f = np.fft.fftn(div[c].reshape(dims).astype(complex))
            psi[c] = np.fft.ifftn(f * inv).real.reshape(-1)
        L.orc_coulomb_apply(grid.pp, _p(np.ascontiguousarray(psi)), _p(grid.U), _p(grid.Unext), _p(grid.E))
        conv.append(s)
        if s < goal:
            break
    return conv


def mirrored_grid(grid: OracleGrid, md):
    """MirroredGrid (OccupationNumbersInTime.java:655-686): dims[md] doubled; each
    cell copied to x and to 2N - 1 - x along md, the mirrored copy's link along
    md taken from the cell at x - 1 (x itself at x = 0)."""
    dims = list(grid.dims)
    n = dims[md]
    dims[md] *= 2
    m = OracleGrid(grid.nc, dims, grid.a, grid.dt, grid.g)
    x = np.indices(grid.dims).reshape(3, -1)
    def idx(pos, dd):
        return (pos[0] * dd[1] + pos[1]) * dd[2] + pos[2]
    i1 = idx(x, dims)
    y = x.copy()
    y[md] = 2 * n - x[md] - 1
    i2 = idx(y, dims)
    z = x.copy()
    z[md] = np.where(z[md] > 0, z[md] - 1, z[md])
    ish = idx(z, grid.dims)
    for k in ("U", "Unext", "E"):
        getattr(m, k)[i1] = getattr(grid, k)
        getattr(m, k)[i2] = getattr(grid, k)
    m.U[i2, md] = grid.U[ish, md]
    return m


def unmirrored_grid(m: OracleGrid, md, dims):
    """UnmirroredGrid (:688-703): the cells of the first half at their own positions."""
    g = OracleGrid(m.nc, dims, m.a, m.dt, m.g)
    x = np.indices(dims).reshape(3, -1)
    im = (x[0] * m.dims[1] + x[1]) * m.dims[2] + x[2]
    for k in ("U", "Unext", "E"):
        getattr(g, k)[...] = getattr(m, k)[im]
    return g


def _su2_pow(u, f):
    """SU2GroupElement.pow(x) = getLink(x getAlgebraElement()) (math/SU2GroupElement.java:234-271,
    math/SU2AlgebraElement.java:140-152), vectorised over the last-but-one axes."""
    norm = np.sqrt(u[..., 1] ** 2 + u[..., 2] ** 2 + u[..., 3] ** 2)
    small = norm < 1e-15
    with np.errstate(invalid="ignore"):
        fac = np.where(small, 2.0, 2.0 * np.arcsin(norm) / np.where(small, 1.0, norm))
    v = u[..., 1:] * fac[..., None] * f[..., None]
    mod = np.sqrt((v ** 2).sum(-1)) / 2
    sinfakt = np.where(mod < 1e-20, 0.0, 0.5 / np.where(mod < 1e-20, 1.0, mod) * np.sin(mod))
    out = np.empty_like(u)
    out[..., 0] = np.cos(mod)
    out[..., 1:] = v * sinfakt[..., None]
    return out


GAUSSIAN, TUKEY, CONE = 1, 2, 4


def windows(g: OracleGrid, flags, time, ctime, cpos, cvel, tukey):
    """GaussianConeRestrictedGrid (:555-599), TukeyConeRestrictedGrid (:601-653)
    and ConeRestrictedGrid (:506-553) in the order calculate applies them
    (:194-202), in place."""
    x = np.indices(g.dims).reshape(3, -1)
    two_sqrt_log_two = 2 * np.sqrt(np.log(2))
    for flag in (GAUSSIAN, TUKEY, CONE):
        if not flags & flag:
            continue
        factor = np.ones(g.V)
        inside = np.ones(g.V, bool)
        for d in range(3):
            if cvel[d] == 0:
                continue
            pos = x[d] * g.a[d]
            min_t, max_t = -abs(time - ctime), abs(time - ctime)
            min_p, max_p = min_t * cvel[d] + cpos[d], max_t * cvel[d] + cpos[d]
            with np.errstate(divide="ignore", invalid="ignore"):
                if flag == GAUSSIAN:
                    sigma = (max_p - min_p) / two_sqrt_log_two
                    factor *= np.exp(-(((pos - cpos[d]) / sigma) ** 2))
                elif flag == TUKEY:
                    xx = (pos - cpos[d]) / (max_p - min_p)
                    w = tukey
                    sup = np.zeros(g.V)
                    m1 = (xx > -.5 - .5 * w) & (xx <= -.5 + .5 * w)
                    m2 = (xx > -.5 + .5 * w) & (xx <= .5 - 0.5 * w)
                    m3 = (xx > 0.5 - 0.5 * w) & (xx < 0.5 + 0.5 * w)
                    sup = np.where(m1, 0.5 * (1 + np.sin(np.pi * (xx + 0.5) / w)), sup)
                    sup = np.where(m2 & ~m1, 1.0, sup)
                    sup = np.where(m3 & ~m1 & ~m2, 0.5 * (1 - np.sin(np.pi * (xx - 0.5) / w)), sup)
                    factor *= sup
                else:
                    inside &= ~((pos < min_p) | (pos > max_p))
        if flag == CONE:
            out = ~inside
            ident = np.zeros(g.U.shape[-1])
            ident[[0, 4, 8] if g.nc == 3 else [0]] = 1.0
            g.U[out] = ident
            g.Unext[out] = ident
            g.E[out] = 0.0
        else:
            g.E *= factor[:, None, None]
            if g.nc == 2:
                f3 = np.repeat(factor[:, None], 3, 1)
                g.U[...] = _su2_pow(g.U, f3)
                g.Unext[...] = _su2_pow(g.Unext, f3)
            else:
                L = lib()
                L.orc_su3_pow.argtypes = [C.c_void_p, C.c_double, C.c_void_p]
                for arr in (g.U, g.Unext):
                    for site in range(g.V):
                        for d in range(3):
                            u = np.ascontiguousarray(arr[site, d])
                            o = np.empty(18)
                            L.orc_su3_pow(_p(u), float(factor[site]), _p(o))
                            arr[site, d] = o


def occupation_numbers(grid: OracleGrid, max_iter=100, goal=1e-18, mirrored_direction=-1, window_flags=0,
                       time=0.0, collision_time=0.0, collision_position=(0.0, 0.0, 0.0),
                       cone_velocity=(0.0, 0.0, 0.0), tukey_width=0.0):
    """OccupationNumbersInTime.calculate on a copy of the grid: returns
    (n [V][3], energy density, divergence list).  Isotropic lattice spacing.
    Options as in the diagnostic's constructor (:92-115); time is the grid's
    time, steps x dt."""
    if mirrored_direction >= 0:
        gm = mirrored_grid(grid, mirrored_direction)
        conv = coulomb_gauge(gm, max_iter, goal)
        g = unmirrored_grid(gm, mirrored_direction, grid.dims)
    else:
        g = grid.copy()
        conv = coulomb_gauge(g, max_iter, goal)
    if window_flags:
        windows(g, window_flags, time, collision_time, collision_position, cone_velocity, tukey_width)
    V, dims = g.V, g.dims
    ncomp = 3 if g.nc == 2 else 8
    a = g.a[0]
    gainv = 1.0 / (a * g.g)
    Ef = np.empty((3, ncomp, V))
    A = np.empty((3, ncomp, V))
    L = lib()
    L.orc_occupation_fields.argtypes = [C.c_void_p] * 4 + [C.c_double, C.c_void_p, C.c_void_p]
    L.orc_occupation_fields(g.pp, _p(g.U), _p(g.Unext), _p(g.E), gainv, _p(Ef), _p(A))
    eF = np.fft.fftn(Ef.reshape(3, ncomp, *dims), axes=(2, 3, 4)).reshape(3, ncomp, V)
    aF = np.fft.fftn(A.reshape(3, ncomp, *dims), axes=(2, 3, 4)).reshape(3, ncomp, V)
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
    n = np.empty((V, ncomp))
    for k in range(ncomp):
        e2 = sum(eF[j, k].real ** 2 + eF[j, k].imag ** 2 for j in range(3))
        a2 = sum(aF[j, k].real ** 2 + aF[j, k].imag ** 2 for j in range(3))
        mixed = -sum(2.0 * (-aF[j, k].imag * eF[j, k].real + aF[j, k].real * eF[j, k].imag) for j in range(3))
        n[:, k] = (e2 + w * w * a2 + w * mixed) * conv_f
    box = np.prod([dims[i] * g.a[i] for i in range(3) if dims[i] > 1])
    energy = n.sum() / (2.0 * box * box)
    return n, energy, conv
