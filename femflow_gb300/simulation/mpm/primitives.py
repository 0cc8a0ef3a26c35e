"""Scene primitives of femflow/simulation/mpm/primitives.py (host-side scene set-up).

Vectorised numpy restatements with the reference's exact conventions:

* ``grid(res)`` (femflow/numerics/geometry.py:100-116): lattice points in [0, 1]^d, first axis
  fastest, a unit axis mapped to 0.
* ``generate_implicit_points`` (primitives.py:46-61) keeps the lattice points whose implicit value,
  which already subtracts ``t``, is larger than ``t`` again (``inside > t``).
* ``generate_cube_points`` (primitives.py:64-76) emits each point as (z, y, x) with x fastest.
"""
from __future__ import annotations

from typing import Callable, Tuple, Union

import numpy as np


def grid(res) -> np.ndarray:
    res = np.asarray(res, dtype=np.int64)
    axes = [np.arange(r, dtype=np.float64) / (1.0 if r == 1 else float(r - 1)) for r in res]
    mesh = np.meshgrid(*axes[::-1], indexing="ij")  # last axis slowest
    return np.stack([m.reshape(-1) for m in mesh[::-1]], axis=1)


def primitive(k: float, t: float, pos: np.ndarray) -> np.ndarray:
    """Schwarz P surface, primitives.py:9-13 (pos: [..., 3])."""
    w = (2.0 * np.pi) / k
    x, y, z = np.moveaxis(np.asarray(pos), -1, 0)
    return np.cos(w * x) + np.cos(w * y) + np.cos(w * z) - t


def gyroid(k: float, t: float, pos: np.ndarray) -> np.ndarray:
    """primitives.py:16-25."""
    w = (2.0 * np.pi) / k
    x, y, z = np.moveaxis(np.asarray(pos), -1, 0)
    return np.sin(w * x) * np.cos(w * y) + np.sin(w * y) * np.cos(w * z) + np.sin(w * z) * np.cos(w * x) - t


def diamond(k: float, t: float, pos: np.ndarray) -> np.ndarray:
    """primitives.py:28-38."""
    w = (2.0 * np.pi) / k
    x, y, z = np.moveaxis(np.asarray(pos), -1, 0)
    sx, sy, sz = np.sin(w * x), np.sin(w * y), np.sin(w * z)
    cx, cy, cz = np.cos(w * x), np.cos(w * y), np.cos(w * z)
    return sx * sy * sz + sx * cy * cz + cx * sy * cz + cx * cy * sz - t


_FNS = {"gyroid": gyroid, "diamond": diamond, "primitive": primitive}


def generate_implicit_points(implicit_fn: Union[Callable, str], k: float, t: float, res: int) -> np.ndarray:
    if isinstance(implicit_fn, str):
        if implicit_fn not in _FNS:
            raise ValueError("Invalid implicit function specified")
        implicit_fn = _FNS[implicit_fn]
    g = grid((res, res, res))
    inside = np.asarray(implicit_fn(k, t, g))
    return g[inside > t]


def generate_cube_points(xb: Tuple[float, float], yb: Tuple[float, float], zb: Tuple[float, float],
                         res: int = 10) -> np.ndarray:
    x = np.linspace(*xb, num=res)
    y = np.linspace(*yb, num=res)
    z = np.linspace(*zb, num=res)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return np.stack([Z.reshape(-1), Y.reshape(-1), X.reshape(-1)], axis=1).astype(np.float64)
