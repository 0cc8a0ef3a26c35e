"""FP64 numpy restatement of the reference's planar colliders — test infrastructure only.

femflow/solvers/mpm/three_d/grid_op.py:50-67 ``check_collision_points(points, normals,
grid_resolution, dx, grid_velocity)``: for each plane (point, normal), normal' = normal +
1/|normal| (line 60, as written; "reference_literal"), and every node I = (i, j, k) with
(I dx - point) . normal' < 0 gets velocity 0.  "sticky" uses normal' = normal, which is what the
evident intent (normal / |normal|) gives for this sign test.  The reference defines no 2D
version; the 2D form here is the same rule on (i, j) nodes.
"""
from __future__ import annotations

import numpy as np


def normal_prime(normal, rule: str = "reference_literal"):
    """normal' of grid_op.py:59-60 (``rule="reference_literal"``) or the normal itself."""
    normal = np.asarray(normal, dtype=np.float64)
    if rule == "reference_literal":
        denom = np.sqrt(np.sum(np.square(normal)))
        return normal + (1.0 / denom)
    if rule == "sticky":
        return normal
    raise ValueError(rule)


def behind(points, normals, grid_resolution, dx, dim: int = 3, rule: str = "reference_literal"):
    """Boolean mask over the (grid_resolution + 1)^dim nodes (C order) behind any of the planes, and
    the per-node signed distances (I dx - point) . normal' of each plane (for margin checks)."""
    R = grid_resolution + 1
    I = np.stack(np.unravel_index(np.arange(R ** dim), (R,) * dim), axis=1).astype(np.float64)
    mask = np.zeros(R ** dim, dtype=bool)
    dots = []
    for point, normal in zip(np.asarray(points, dtype=np.float64), np.asarray(normals, dtype=np.float64)):
        n1 = normal_prime(normal, rule)
        offset = I * dx - point
        # the sum is taken term by term in index order, as numpy's dot of two short vectors
        dot = offset[:, 0] * n1[0]
        for d in range(1, dim):
            dot = dot + offset[:, d] * n1[d]
        dots.append(dot)
        mask |= dot < 0
    return mask, np.array(dots)


def check_collision_points(points, normals, grid_resolution, dx, grid_velocity, rule: str = "reference_literal"):
    """In place on grid_velocity [R, R, R, 3] (or [R, R, 2] in 2D), as grid_op.py:50-67."""
    dim = grid_velocity.ndim - 1
    mask, _ = behind(points, normals, grid_resolution, dx, dim, rule)
    flat = grid_velocity.reshape(-1, grid_velocity.shape[-1])
    flat[mask] = 0.0
    return grid_velocity
