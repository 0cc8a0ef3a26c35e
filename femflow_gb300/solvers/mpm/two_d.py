"""Mirror of ``femflow.solvers.mpm.two_d`` (femflow/solvers/mpm/two_d/{p2g,grid_op,g2p}.py).

Scalar ``mass``, ``mu_0`` and ``lambda_0`` as in two_d/p2g.py:11-29; positions are an ``x[N,2]``
array.  The stored F is the reference's up to sign: two_d/g2p.py:37-43 rebuilds F from an SVD
whose sign convention is LAPACK's, and every observable (x, v, C, F F^T, det F) is unchanged by
that sign.
"""
from __future__ import annotations

import ctypes

from ... import _native as N
from ... import engine as E
from . import _phase as P


def p2g(inv_dx, hardening, mu_0, lambda_0, mass, dx, dt, volume, grid_velocity, grid_mass, x, v, F, C, Jp,
        model: str = "neo_hookean", *, deterministic: bool = False):
    """two_d/p2g.py:11-76 (``deterministic=True``: fixed summation order, bit-identical runs)."""
    dtype = P.dtype_of(x, v, grid_velocity)
    st = E.stage([x, v, F, C, Jp, grid_velocity, grid_mass], dtype=dtype)
    xx, vv, FF, CC, JJ, gv, gm = st.dev
    E.check_tensors(dtype, xx, vv, FF, CC, JJ, gv, gm)
    res = gv.shape[0] - 1
    prm = E.make_params(2, res, dtype, dx, inv_dx, dt, 0.0, volume, hardening, mass, mu_0, lambda_0, model=model,
                        deterministic=deterministic)
    ps = E.particles_struct(xx, vv, FF, CC, JJ)
    g = E.grid_struct(gv, gm)
    P.run("ffmpm_p2g", prm, ps.n, xx.device, ctypes.byref(prm), ctypes.byref(ps), ctypes.byref(g))
    st.write_back([5, 6])


def grid_op(grid_resolution, dt, gravity, grid_velocity, grid_mass, wall_mode: str = "reference"):
    """two_d/grid_op.py:5-24 (no dx argument, as the reference)."""
    dtype = P.dtype_of(grid_velocity)
    st = E.stage([grid_velocity, grid_mass], dtype=dtype)
    gv, gm = st.dev
    E.check_tensors(dtype, gv, gm)
    prm = E.make_params(2, grid_resolution, dtype, 1.0 / grid_resolution, grid_resolution, dt, gravity,
                        wall_mode=wall_mode)
    g = E.grid_struct(gv, gm)
    N.call("ffmpm_grid_op", ctypes.byref(prm), ctypes.byref(g), P.stream(gv.device))
    st.write_back([0])


def g2p(inv_dx, dt, grid_velocity, x, v, F, C, Jp, model: str = "neo_hookean"):
    """two_d/g2p.py:5-47."""
    dtype = P.dtype_of(x, v, grid_velocity)
    st = E.stage([x, v, F, C, Jp, grid_velocity], dtype=dtype)
    xx, vv, FF, CC, JJ, gv = st.dev
    E.check_tensors(dtype, xx, vv, FF, CC, JJ, gv)
    res = gv.shape[0] - 1
    prm = E.make_params(2, res, dtype, 1.0 / inv_dx, inv_dx, dt, model=model)
    ps = E.particles_struct(xx, vv, FF, CC, JJ)
    g = E.grid_struct(gv, None)
    P.run("ffmpm_g2p", prm, ps.n, xx.device, ctypes.byref(prm), ctypes.byref(g), ctypes.byref(ps))
    st.write_back([0, 1, 2, 3, 4])


def solve_mls_mpm_2d(res, inv_dx, hardening, mu_0, lambda_0, mass, dx, dt, volume, gravity, x, v, F, C, Jp,
                     model: str = "neo_hookean", wall_mode: str = "reference", *, deterministic: bool = False):
    """One 2D substep: the p2g -> grid_op -> g2p sequence on a fresh grid, fused on the GPU.

    The reference has no 2D driver; this is the call sequence of mls_mpm.py:54-79 with the
    two_d functions, with the grid held in the workspace instead of the caller's arrays.
    """
    dtype = P.dtype_of(x, v)
    st = E.stage([x, v, F, C, Jp], dtype=dtype)
    xx, vv, FF, CC, JJ = st.dev
    E.check_tensors(dtype, xx, vv, FF, CC, JJ)
    prm = E.make_params(2, res, dtype, dx, inv_dx, dt, gravity, volume, hardening, mass, mu_0, lambda_0,
                        model=model, wall_mode=wall_mode, deterministic=deterministic)
    ps = E.particles_struct(xx, vv, FF, CC, JJ)
    P.run("ffmpm_substep", prm, ps.n, xx.device, ctypes.byref(prm), ctypes.byref(ps))
    st.write_back([0, 1, 2, 3, 4])
