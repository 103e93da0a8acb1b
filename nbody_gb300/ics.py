"""Seeded synthetic initial conditions for the FMM step.

These stand in for the workloads the step is measured on (there is no public
data set): Plummer spheres sampled with the Aarseth, Henon & Wielen (1974)
method, a uniform cube with log-normal masses, a head-on collision of two
Plummer spheres and a clustered set of Plummer sub-clusters.  Every generator
takes a seed and returns float64 arrays ``pos (n,3), vel (n,3), mass (n,)``;
charge = mass for gravity (the reference couples through ``charge`` and
integrates with ``mass``, src/field.cl:27-29, src/open_cl_simulation.cpp:605).
"""
from __future__ import annotations

import numpy as np

__all__ = ["plummer", "uniform_cube", "collision", "clustered", "workload"]


def _isotropic(rng, n):
    z = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(1.0 - z * z)
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], axis=1)


def plummer(n, a=1.0, total_mass=1.0, G=1.0, rmax=20.0, seed=0, centre=True):
    """Plummer sphere, radii truncated at ``rmax`` * a, isotropic DF velocities.

    Radii invert the cumulative mass M(r)/M = r^3/(r^2+a^2)^(3/2); speeds are
    q * v_esc with q drawn from g(q) = q^2 (1-q^2)^(7/2) by rejection
    (Aarseth, Henon & Wielen 1974).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    r = np.empty(0)
    while r.size < n:
        x1 = rng.uniform(1e-10, 1.0, 2 * n)
        rr = a / np.sqrt(x1 ** (-2.0 / 3.0) - 1.0)
        r = np.concatenate([r, rr[rr <= rmax * a]])
    r = r[:n]
    pos = r[:, None] * _isotropic(rng, n)
    ve = np.sqrt(2.0 * G * total_mass / a) * (1.0 + (r / a) ** 2) ** -0.25
    q = np.empty(0)
    while q.size < n:
        x4 = rng.uniform(0.0, 1.0, 2 * n)
        x5 = rng.uniform(0.0, 1.0, 2 * n)
        ok = 0.1 * x5 < x4 * x4 * (1.0 - x4 * x4) ** 3.5
        q = np.concatenate([q, x4[ok]])
    q = q[:n]
    vel = (q * ve)[:, None] * _isotropic(rng, n)
    mass = np.full(n, total_mass / n)
    if centre and n > 0:
        pos -= np.average(pos, axis=0, weights=mass)
        vel -= np.average(vel, axis=0, weights=mass)
    return pos, vel, mass


def uniform_cube(n, seed=0, sigma=0.5):
    """Uniform in [0,1)^3, log-normal(0, sigma) masses normalised to 1, v = 0."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.uniform(0.0, 1.0, (n, 3))
    mass = rng.lognormal(0.0, sigma, n)
    mass /= mass.sum()
    return pos, np.zeros((n, 3)), mass


def collision(n, separation=10.0, impact=1.0, speed=0.5, seed=0):
    """Two equal Plummer spheres (a=1, mass 0.5 each) approaching head-on.

    Centres ``separation`` apart on x, offset by ``impact`` in y, relative
    speed ``speed`` along x.
    """
    h = n // 2
    p1, v1, m1 = plummer(h, total_mass=0.5, seed=seed)
    p2, v2, m2 = plummer(n - h, total_mass=0.5, seed=seed + 7919)
    off = np.array([separation / 2.0, impact / 2.0, 0.0])
    dv = np.array([speed / 2.0, 0.0, 0.0])
    pos = np.concatenate([p1 - off, p2 + off])
    vel = np.concatenate([v1 + dv, v2 - dv])
    return pos, vel, np.concatenate([m1, m2])


def clustered(n, nclusters=64, scale=0.05, seed=0):
    """Plummer sub-clusters (scale radius ``scale``) placed on a Plummer a=1.

    Body masses follow dN/dM ~ M^-2 on [1,100] (inverse-CDF sampling),
    normalised to a total of 1; each sub-cluster gets its share of bodies,
    internal DF velocities for its own mass, and the DF velocity of its centre.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    cpos, cvel, _ = plummer(nclusters, seed=seed + 1)
    counts = np.full(nclusters, n // nclusters)
    counts[: n - counts.sum()] += 1
    u = rng.uniform(0.0, 1.0, n)
    mass = 1.0 / (1.0 - u * (1.0 - 1.0 / 100.0))     # inverse CDF of M^-2 on [1, 100]
    mass /= mass.sum()
    pos = np.empty((n, 3))
    vel = np.empty((n, 3))
    o = 0
    for c in range(nclusters):
        k = counts[c]
        mc = mass[o:o + k].sum()
        p, v, _ = plummer(k, a=scale, total_mass=mc, seed=seed + 100 + c)
        pos[o:o + k] = p + cpos[c]
        vel[o:o + k] = v + cvel[c]
        o += k
    return pos, vel, mass


def workload(name, n=None, seed=0):
    """Named workloads with their default sizes.

    plummer4k   N=4,096 Plummer (eps 0.01, dt 1e-3, theta 0.5, capacity 16)
    cube256k    N=262,144 uniform cube, log-normal masses (eps 1e-3, capacity 32)
    collision1m N=1,048,576 two-Plummer collision (eps 0.005, dt 5e-4)
    plummer64k  N=65,536 Plummer (eps 0.01, dt 1e-3)
    clusters4m  N=4,194,304 in 64 sub-clusters (eps 1e-3, dt 2.5e-4)
    """
    if name == "plummer4k":
        return plummer(n or 4096, seed=seed)
    if name == "cube256k":
        return uniform_cube(n or 262144, seed=seed)
    if name == "collision1m":
        return collision(n or 1048576, seed=seed)
    if name == "plummer64k":
        return plummer(n or 65536, seed=seed)
    if name == "clusters4m":
        return clustered(n or 4194304, seed=seed)
    raise KeyError(name)
