#!/usr/bin/env python3
"""Writes the golden fixtures of this directory from the CPU oracle.

The reference ships no golden trajectories (its tests are property tests), so
these fixtures are the oracle's own seeded outputs: they pin the oracle
against regressions (tests/test_golden.py regenerates them on the CPU) and
serve as the fixed reference of the GPU parity tests (tests/test_gpu_golden.py).
Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def pure_ym(nc, dims, seed, sigma, steps, dt=0.05, a=(1.0, 1.0, 1.0), g=1.0):
    """Seeded links and E, E projected onto Gauss's law, Simulation.initialize,
    then `steps` x Simulation.step with BulkQuantities after every step."""
    import oracle
    o = oracle.OracleGrid(nc, dims, a=a, dt=dt, g=g)
    o.random_links(seed, sigma)
    o.random_e(seed, sigma)
    o.gauss_project(tol_g2=1e-26)
    U0, E0 = o.U.copy(), o.E.copy()
    sim = oracle.OracleSimulation(o)
    sim.initialize()
    bulk = []
    for _ in range(steps):
        sim.step()
        bulk.append(o.bulk())
    return dict(nc=nc, dims=np.array(dims), a=np.array(a), dt=dt, g=g, seed=seed, sigma=sigma, steps=steps,
                U0=U0, E0=E0, U=o.U.copy(), Unext=o.Unext.copy(), E=o.E.copy(), bulk=np.array(bulk),
                energy_density=o.energy_density(), projected0=o.projected_energy(0))


def cpic(dims, n, seed, steps, dt=0.5):
    """Random links and particles (NGP, along all three axes, some starting on
    half-integer positions), Simulation.initialize and `steps` coupled steps."""
    import oracle
    nc = 2
    o = oracle.OracleGrid(nc, dims, dt=dt)
    o.random_links(seed, 0.4)
    o.random_e(seed, 0.2)
    rng = np.random.default_rng(seed)
    P = oracle.OracleParticles(nc, n)
    P.dir[:] = rng.choice([0, 0, 1, 2], n)
    sign = rng.choice([-1.0, 1.0], n)
    for k in range(n):
        P.vel[k, P.dir[k]] = sign[k]
    P.pos0[:] = rng.uniform(0, 1, (n, 3)) * np.array(dims)
    ties = rng.random(n) < 0.25
    P.pos0[ties] = np.floor(P.pos0[ties]) + 0.5
    P.pos1[:] = P.pos0 - P.vel * dt
    P.Q0[:] = rng.normal(0, 0.3, (n, 3))
    P.Q1[:] = P.Q0
    init = {k: getattr(P, k).copy() for k in ("pos0", "pos1", "vel", "Q0", "Q1", "dir")}
    U0, E0 = o.U.copy(), o.E.copy()
    sim = oracle.OracleSimulation(o, P)
    sim.initialize()
    for _ in range(steps):
        sim.step()
    out = dict(nc=nc, dims=np.array(dims), dt=dt, seed=seed, steps=steps, U0=U0, E0=E0,
               U=o.U.copy(), E=o.E.copy(), rho=o.rho.copy(), J=o.J.copy())
    out.update({"p_" + k: v for k, v in init.items()})
    out.update({"P_" + k: getattr(P, k).copy() for k in ("pos0", "pos1", "Q0", "Q1")})
    return out


def cgc(dims, steps, dt=0.5):
    """Two MV nuclei (the CPIC collision setup on a small lattice), the particle
    list they create, and `steps` coupled steps with the ProjectedEnergyDensity
    rows (energy and Poynting) at the end."""
    import oracle
    from oracle import cgc as ocgc
    o = oracle.OracleGrid(2, dims, dt=dt)
    nuclei = [ocgc.MVNucleus(orientation=1, location=6.0, width=1.5, mu=0.5, seed=1),
              ocgc.MVNucleus(orientation=-1, location=14.0, width=1.5, mu=0.5, seed=2)]
    P, _ = ocgc.cgc_mv(o, nuclei)
    out = dict(dims=np.array(dims), dt=dt, steps=steps, ic_U=o.U.copy(), ic_Unext=o.Unext.copy(), ic_E=o.E.copy(),
               ic_pos0=P.pos0.copy(), ic_pos1=P.pos1.copy(), ic_Q0=P.Q0.copy())
    sim = oracle.OracleSimulation(o, P)
    sim.initialize()
    for _ in range(steps):
        sim.step()
    out.update(U=o.U.copy(), E=o.E.copy(), P_pos0=P.pos0.copy(), P_Q0=P.Q0.copy(),
               projected=o.projected_energy(0), poynting=o.projected_poynting(0), bulk=o.bulk())
    return out


CASES = {
    "su2_fp64_6cube": lambda: pure_ym(2, (6, 6, 6), 11, 0.2, 20),
    "su3_fp64_4x4x6": lambda: pure_ym(3, (4, 4, 6), 12, 0.2, 10, a=(1.0, 1.0, 0.8)),
    "cpic_su2_12x6x6": lambda: cpic((12, 6, 6), 300, 13, 8),
    "cgc_su2_20x6x6": lambda: cgc((20, 6, 6), 6),
}


def main():
    for name, make in CASES.items():
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **make())
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
