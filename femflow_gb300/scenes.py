"""Seeded synthetic particle scenes used by the benchmark, the profiler driver and the tests."""
from __future__ import annotations

import numpy as np


def lame(E: float, nu: float):
    """(mu, lambda) from Young's modulus and Poisson ratio (femflow/numerics/fem.py:1-6)."""
    return E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))


def two_cubes(n_per_cube: int = 524_288, edge: float = 0.2, speed: float = 1.0, E: float = 4.5e3, nu: float = 0.3,
              rho: float = 1.0, seed: int = 0, centres=((0.35, 0.5, 0.5), (0.65, 0.5, 0.5))) -> dict:
    """Two seeded-uniform cubes moving toward each other along x (+speed / -speed).

    Particle volume = total cube volume / N and mass = rho * volume (uniform material).
    """
    rng = np.random.default_rng(seed)
    a = rng.uniform(-edge / 2, edge / 2, (n_per_cube, 3)) + np.asarray(centres[0])
    b = rng.uniform(-edge / 2, edge / 2, (n_per_cube, 3)) + np.asarray(centres[1])
    x = np.concatenate([a, b])
    n = len(x)
    v = np.zeros((n, 3))
    v[:n_per_cube, 0], v[n_per_cube:, 0] = speed, -speed
    vol = 2 * edge ** 3 / n
    mu, lam = lame(E, nu)
    return dict(x=x, v=v, n=n, vol=vol, mass=rho * vol, mu=mu, lam=lam, E=E, nu=nu)


def block_2d(n: int, lo=(0.3, 0.4), hi=(0.6, 0.7), E: float = 1e4, nu: float = 0.2, rho: float = 1.0,
             seed: int = 0) -> dict:
    """A seeded-uniform rectangle of particles at rest (the 2D block-drop scene)."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(lo, hi, size=(n, 2))
    vol = (hi[0] - lo[0]) * (hi[1] - lo[1]) / n
    mu, lam = lame(E, nu)
    return dict(x=x, v=np.zeros((n, 2)), n=n, vol=vol, mass=rho * vol, mu=mu, lam=lam, E=E, nu=nu)
