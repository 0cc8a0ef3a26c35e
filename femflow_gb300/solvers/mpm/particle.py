"""Particle records (femflow/solvers/mpm/particle.py:10-33).

``Particle`` keeps the reference's per-particle record for code that builds lists of them.
``ParticleSet`` is the structure-of-arrays form the kernels use: ``pos [N,3]`` plus per-particle
``mass``, ``mu_0``, ``lambda_0`` (``force`` is carried for compatibility; the reference never
reads it).
"""
from __future__ import annotations

from typing import List

import numpy as np
import torch


class Particle:
    """One particle: ``Particle(pos, force, mass, lambda_, mu)`` (particle.py:18-25 argument order)."""

    def __init__(self, pos, force: float, mass: float, lambda_: float, mu: float):
        self.pos = np.asarray(pos, dtype=np.float64)
        self.force = float(force)
        self.mass = float(mass)
        self.lambda_0 = float(lambda_)
        self.mu_0 = float(mu)


class ParticleSet:
    """Particles as tensors (any device; CUDA tensors avoid host staging)."""

    def __init__(self, pos: torch.Tensor, mass: torch.Tensor, mu_0: torch.Tensor, lambda_0: torch.Tensor,
                 force: torch.Tensor | None = None):
        n = pos.shape[0]
        for name, t in (("mass", mass), ("mu_0", mu_0), ("lambda_0", lambda_0)):
            if t.shape[0] != n:
                raise ValueError(f"{name} has {t.shape[0]} entries for {n} particles")
        self.pos, self.mass, self.mu_0, self.lambda_0 = pos, mass, mu_0, lambda_0
        self.force = force

    def __len__(self):
        return self.pos.shape[0]

    @classmethod
    def from_particles(cls, particles: List[Particle], dtype=torch.float64, device="cpu") -> "ParticleSet":
        pos = torch.tensor(np.array([p.pos for p in particles]), dtype=dtype, device=device)
        f = lambda attr: torch.tensor([getattr(p, attr) for p in particles], dtype=dtype, device=device)
        return cls(pos, f("mass"), f("mu_0"), f("lambda_0"), f("force"))

    def write_positions(self, particles: List[Particle]):
        pos = self.pos.detach().cpu().numpy().astype(np.float64)
        for p, row in zip(particles, pos):
            p.pos[...] = row


def map_particles_to_pos(particles, coeff: float) -> np.ndarray:
    """Flattened positions divided by ``coeff`` (particle.py:30-33)."""
    if isinstance(particles, ParticleSet):
        return (particles.pos.detach().double().cpu().numpy() / coeff).reshape(-1)
    return (np.array([p.pos.copy() / coeff for p in particles])).reshape(-1)
