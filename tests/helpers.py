"""Shared test helpers: seeded initial conditions from the oracle and error metrics."""
import functools

import numpy as np


@functools.lru_cache(maxsize=8)
def oracle_ic(nc, dims, seed, sigma_a, sigma_e, dt=0.05, a=(1.0, 1.0, 1.0)):
    """Seeded links/E (the oracle's counter-based generator), E projected onto Gauss's law."""
    import oracle
    g = oracle.OracleGrid(nc, dims, a=a, dt=dt)
    g.random_links(seed, sigma_a)
    g.random_e(seed, sigma_e)
    it, g2 = g.gauss_project(tol_g2=1e-26)
    assert g2 < 1e-24, g2
    return g


def fresh(g):
    return g.copy()


def link_rel_err(a, b):
    """max over links of |a - b| / |b| (links have unit norm scale)."""
    d = np.linalg.norm((a - b).reshape(a.shape[0] * a.shape[1], -1), axis=1)
    n = np.linalg.norm(b.reshape(b.shape[0] * b.shape[1], -1), axis=1)
    return float(np.max(d / np.maximum(n, 1e-300)))


def field_rel_err(a, b):
    """max over links of |a - b| / max(|b|, rms(b)): relative per link, with the
    lattice rms as the floor so that nearly vanishing links do not dominate."""
    fa = a.reshape(-1, a.shape[-1])
    fb = b.reshape(-1, b.shape[-1])
    d = np.linalg.norm(fa - fb, axis=1)
    n = np.linalg.norm(fb, axis=1)
    rms = np.sqrt(np.mean(n ** 2))
    return float(np.max(d / np.maximum(n, rms)))


def to_gen(orc, nc, E):
    """Reference-layout algebra field -> generator components (SU3AlgebraElement.get)."""
    if nc == 2:
        return E.copy()
    flat = E.reshape(-1, 9)
    out = np.empty((flat.shape[0], 8))
    for k in range(flat.shape[0]):
        out[k] = orc.alg_to_gen(3, flat[k])
    return out.reshape(E.shape[:-1] + (8,))
