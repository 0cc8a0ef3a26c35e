"""Mirror of ``femflow.solvers.mpm.three_d`` (femflow/solvers/mpm/three_d/{p2g,grid_op,g2p}.py).

Same arguments and in-place semantics as the numba functions; arrays may be CUDA tensors (no
copies) or host arrays (numpy / CPU tensors, staged to the GPU and written back).  An
out-of-grid particle raises ``RuntimeError`` as the reference does (utils.py:138-150).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ... import _native as N
from ... import engine as E
from . import _phase as P


def p2g(inv_dx, hardening, dx, dt, volume, grid_velocity, grid_mass, particles, v, F, C, Jp,
        model: str = "neo_hookean", *, deterministic: bool = False):
    """three_d/p2g.py:14-80: add the particles' momentum and mass into the grid.

    ``deterministic=True`` sums every node in a fixed order (bit-identical across runs).
    """
    pset, plist = P.split_particles(particles)
    dtype = P.dtype_of(v, F, grid_velocity)
    st = E.stage([pset.pos, pset.mass, pset.mu_0, pset.lambda_0, v, F, C, Jp, grid_velocity, grid_mass], dtype=dtype)
    x, m, mu, lam, vv, FF, CC, JJ, gv, gm = st.dev
    E.check_tensors(dtype, x, m, mu, lam, vv, FF, CC, JJ, gv, gm)
    res = gv.shape[0] - 1
    prm = E.make_params(3, res, dtype, dx, inv_dx, dt, 0.0, volume, hardening, model=model,
                        deterministic=deterministic)
    ps = E.particles_struct(x, vv, FF, CC, JJ, m, mu, lam)
    g = E.grid_struct(gv, gm)
    P.run("ffmpm_p2g", prm, ps.n, x.device, ctypes.byref(prm), ctypes.byref(ps), ctypes.byref(g))
    st.write_back([8, 9])


def grid_op(grid_resolution, dx, dt, gravity, grid_velocity, grid_mass):
    """three_d/grid_op.py:5-47: momentum -> velocity, gravity, clamp to 0.9 dx/dt, slip walls."""
    dtype = P.dtype_of(grid_velocity)
    st = E.stage([grid_velocity, grid_mass], dtype=dtype)
    gv, gm = st.dev
    E.check_tensors(dtype, gv, gm)
    prm = E.make_params(3, grid_resolution, dtype, dx, 1.0 / dx, dt, gravity)
    g = E.grid_struct(gv, gm)
    N.call("ffmpm_grid_op", ctypes.byref(prm), ctypes.byref(g), P.stream(gv.device))
    st.write_back([0])


def g2p(inv_dx, dt, grid_velocity, particles, v, F, C, Jp, model: str = "neo_hookean"):
    """three_d/g2p.py:9-59: gather v and APIC C, advect, F <- (I + dt C) F."""
    pset, plist = P.split_particles(particles)
    dtype = P.dtype_of(v, F, grid_velocity)
    st = E.stage([pset.pos, v, F, C, Jp, grid_velocity], dtype=dtype)
    x, vv, FF, CC, JJ, gv = st.dev
    E.check_tensors(dtype, x, vv, FF, CC, JJ, gv)
    res = gv.shape[0] - 1
    prm = E.make_params(3, res, dtype, 1.0 / inv_dx, inv_dx, dt, model=model)
    ps = E.particles_struct(x, vv, FF, CC, JJ)
    g = E.grid_struct(gv, None)
    P.run("ffmpm_g2p", prm, ps.n, x.device, ctypes.byref(prm), ctypes.byref(g), ctypes.byref(ps))
    st.write_back([0, 1, 2, 3, 4])
    if plist is not None:
        pset.write_positions(plist)


def check_collision_points(points, normals, grid_resolution, dx, grid_velocity, rule: str = "reference_literal"):
    """three_d/grid_op.py:50-67: for every plane (point, normal) and every grid node I, zero the
    node's velocity where (I dx - point) . normal' < 0, in place on the caller's grid.

    ``rule="reference_literal"`` (default, the reference's behaviour) uses normal' = normal +
    1/|normal| exactly as line 60 writes it, which tilts the plane; ``rule="sticky"`` uses the
    normal itself (what normalising would give, the evident intent).  The solvers take planes
    through ``planes=`` instead and apply them inside every grid update.
    """
    points = np.asarray(points.cpu() if isinstance(points, torch.Tensor) else points, dtype=np.float64).reshape(-1, 3)
    normals = np.asarray(normals.cpu() if isinstance(normals, torch.Tensor) else normals,
                         dtype=np.float64).reshape(-1, 3)
    if points.shape != normals.shape:
        raise ValueError("points and normals differ in length")
    dtype = P.dtype_of(grid_velocity)
    st = E.stage([grid_velocity], dtype=dtype)
    (gv,) = st.dev
    E.check_tensors(dtype, gv)
    prm = E.make_params(3, grid_resolution, dtype, dx, 1.0 / dx, 1.0, plane_rule=rule)
    pts = np.ascontiguousarray(points)
    nrm = np.ascontiguousarray(normals)
    N.call("ffmpm_check_collision_points", ctypes.byref(prm), pts.ctypes.data_as(ctypes.c_void_p),
           nrm.ctypes.data_as(ctypes.c_void_p), int(len(pts)), ctypes.c_void_p(gv.data_ptr()), P.stream(gv.device))
    st.write_back([0])
