"""FP64 CPU oracle of the MLS-MPM substep — test infrastructure, never the product path.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` import this
package.  It wraps ``mpm_oracle.c`` (a serial C restatement of FEMFlow's
``femflow/solvers/mpm/{two_d,three_d}/*.py`` and ``utils.py``) through ctypes on numpy float64
arrays, with the reference's own argument order and in-place semantics:

* ``p2g_3d``      ~ ``three_d.p2g``     (femflow/solvers/mpm/three_d/p2g.py:14-80)
* ``grid_op_3d``  ~ ``three_d.grid_op`` (femflow/solvers/mpm/three_d/grid_op.py:5-47)
* ``g2p_3d``      ~ ``three_d.g2p``     (femflow/solvers/mpm/three_d/g2p.py:9-59)
* ``substep_3d``  ~ ``solve_mls_mpm_3d`` (femflow/solvers/mpm/mls_mpm.py:40-79)
* ``p2g_2d`` / ``grid_op_2d`` / ``g2p_2d`` / ``substep_2d`` ~ ``two_d.*``

Out-of-bounds particles raise ``RuntimeError`` as the reference does (utils.py:138-150).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle_mpm.so")
_lib = None

MODELS = {"neo_hookean": 0, "snow": 1, "fixed_corotated": 2}

_dp = ctypes.POINTER(ctypes.c_double)
_d = ctypes.c_double
_i = ctypes.c_int
_i64 = ctypes.c_int64


def build(force: bool = False) -> str:
    """Compile mpm_oracle.c with the Makefile beside it; returns the library path."""
    src = os.path.join(_HERE, "mpm_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "-B"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.orc_p2g_3d.argtypes = [_d, _d, _d, _d, _d, _i, _dp, _dp, _i64, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _i]
        L.orc_grid_op_3d.argtypes = [_i, _d, _d, _d, _dp, _dp]
        L.orc_g2p_3d.argtypes = [_d, _d, _i, _dp, _i64, _dp, _dp, _dp, _dp, _dp, _i]
        L.orc_substep_3d.argtypes = [_i, _d, _d, _d, _d, _d, _d, _i64, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _i]
        L.orc_substep_3d_par.argtypes = [_i, _d, _d, _d, _d, _d, _d, _i64, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                         _i, _i, _dp]
        L.orc_p2g_2d.argtypes = [_d, _d, _d, _d, _d, _d, _d, _d, _i, _dp, _dp, _i64, _dp, _dp, _dp, _dp, _dp, _i]
        L.orc_grid_op_2d.argtypes = [_i, _d, _d, _dp, _dp]
        L.orc_g2p_2d.argtypes = [_d, _d, _i, _dp, _i64, _dp, _dp, _dp, _dp, _dp, _i]
        L.orc_substep_2d.argtypes = [_i, _d, _d, _d, _d, _d, _d, _d, _d, _d, _i64, _dp, _dp, _dp, _dp, _dp, _i]
        L.orc_bspline_weights.argtypes = [_d, _dp]
        L.orc_polar_3d.argtypes = [_dp, _dp]
        L.orc_polar_2d.argtypes = [_dp, _dp]
        L.orc_svd_3d.argtypes = [_dp, _dp, _dp, _dp]
        L.orc_stress_affine_3d.argtypes = [_dp, _d, _d, _d, _d, _d, _d, _dp, _dp]
        L.orc_stress_affine_2d.argtypes = [_dp, _d, _d, _d, _d, _d, _d, _dp, _dp]
        L.orc_num_threads.restype = _i
        _lib = L
    return _lib


def _p(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("oracle arrays must be C-contiguous float64")
    return a.ctypes.data_as(_dp)


def _check(status: int):
    if status == 1:
        raise RuntimeError("particle out of grid bounds")
    if status != 0:
        raise RuntimeError(f"oracle error {status}")


def _model(model) -> int:
    return MODELS[model] if isinstance(model, str) else int(model)


# ---------------------------------------------------------------- 3D
def p2g_3d(inv_dx, hardening, dx, dt, volume, grid_velocity, grid_mass, x, mass, mu_0, lambda_0,
           v, F, C, Jp, model="neo_hookean"):
    res = grid_velocity.shape[0] - 1
    _check(lib().orc_p2g_3d(inv_dx, hardening, dx, dt, volume, res, _p(grid_velocity), _p(grid_mass),
                            x.shape[0], _p(x), _p(mass), _p(mu_0), _p(lambda_0), _p(v), _p(F), _p(C),
                            _p(Jp), _model(model)))


def grid_op_3d(grid_resolution, dx, dt, gravity, grid_velocity, grid_mass):
    _check(lib().orc_grid_op_3d(grid_resolution, dx, dt, gravity, _p(grid_velocity), _p(grid_mass)))


def g2p_3d(inv_dx, dt, grid_velocity, x, v, F, C, Jp, model="neo_hookean"):
    res = grid_velocity.shape[0] - 1
    _check(lib().orc_g2p_3d(inv_dx, dt, res, _p(grid_velocity), x.shape[0], _p(x), _p(v), _p(F), _p(C),
                            _p(Jp), _model(model)))


def substep_3d(res, inv_dx, hardening, dx, dt, volume, gravity, x, mass, mu_0, lambda_0, v, F, C, Jp,
               model="neo_hookean"):
    _check(lib().orc_substep_3d(res, inv_dx, hardening, dx, dt, volume, gravity, x.shape[0], _p(x),
                                _p(mass), _p(mu_0), _p(lambda_0), _p(v), _p(F), _p(C), _p(Jp),
                                _model(model)))


def substep_3d_par(res, inv_dx, hardening, dx, dt, volume, gravity, x, mass, mu_0, lambda_0, v, F, C, Jp,
                   model="neo_hookean", nthreads=0, grid_scratch=None):
    """Multi-threaded timing variant (OpenMP, atomic scatter): not a parity reference."""
    gs = _p(grid_scratch) if grid_scratch is not None else None
    _check(lib().orc_substep_3d_par(res, inv_dx, hardening, dx, dt, volume, gravity, x.shape[0], _p(x),
                                    _p(mass), _p(mu_0), _p(lambda_0), _p(v), _p(F), _p(C), _p(Jp),
                                    _model(model), nthreads, gs))


def num_threads() -> int:
    return int(lib().orc_num_threads())


# ---------------------------------------------------------------- 2D
def p2g_2d(inv_dx, hardening, mu_0, lambda_0, mass, dx, dt, volume, grid_velocity, grid_mass, x, v, F, C,
           Jp, model="neo_hookean"):
    res = grid_velocity.shape[0] - 1
    _check(lib().orc_p2g_2d(inv_dx, hardening, mu_0, lambda_0, mass, dx, dt, volume, res, _p(grid_velocity),
                            _p(grid_mass), x.shape[0], _p(x), _p(v), _p(F), _p(C), _p(Jp), _model(model)))


def grid_op_2d(grid_resolution, dt, gravity, grid_velocity, grid_mass):
    _check(lib().orc_grid_op_2d(grid_resolution, dt, gravity, _p(grid_velocity), _p(grid_mass)))


def g2p_2d(inv_dx, dt, grid_velocity, x, v, F, C, Jp, model="neo_hookean"):
    res = grid_velocity.shape[0] - 1
    _check(lib().orc_g2p_2d(inv_dx, dt, res, _p(grid_velocity), x.shape[0], _p(x), _p(v), _p(F), _p(C),
                            _p(Jp), _model(model)))


def substep_2d(res, inv_dx, hardening, mu_0, lambda_0, mass, dx, dt, volume, gravity, x, v, F, C, Jp,
               model="neo_hookean"):
    _check(lib().orc_substep_2d(res, inv_dx, hardening, mu_0, lambda_0, mass, dx, dt, volume, gravity,
                                x.shape[0], _p(x), _p(v), _p(F), _p(C), _p(Jp), _model(model)))


# ---------------------------------------------------------------- helpers (known-answer tests)
def bspline_weights(fx: float) -> np.ndarray:
    w = np.zeros(3)
    lib().orc_bspline_weights(fx, _p(w))
    return w


def polar_3d(F: np.ndarray) -> np.ndarray:
    F = np.ascontiguousarray(F, dtype=np.float64)
    R = np.zeros((3, 3))
    lib().orc_polar_3d(_p(F), _p(R))
    return R


def polar_2d(F: np.ndarray) -> np.ndarray:
    F = np.ascontiguousarray(F, dtype=np.float64)
    R = np.zeros((2, 2))
    lib().orc_polar_2d(_p(F), _p(R))
    return R


def svd_3d(F: np.ndarray):
    F = np.ascontiguousarray(F, dtype=np.float64)
    U, s, V = np.zeros((3, 3)), np.zeros(3), np.zeros((3, 3))
    lib().orc_svd_3d(_p(F), _p(U), _p(s), _p(V))
    return U, s, V


def stress_affine_3d(F, inv_dx, mu, lam, dt, vol, mass, C) -> np.ndarray:
    F = np.ascontiguousarray(F, dtype=np.float64)
    C = np.ascontiguousarray(C, dtype=np.float64)
    A = np.zeros((3, 3))
    lib().orc_stress_affine_3d(_p(F), inv_dx, mu, lam, dt, vol, mass, _p(C), _p(A))
    return A


def stress_affine_2d(F, inv_dx, mu, lam, dt, vol, mass, C) -> np.ndarray:
    F = np.ascontiguousarray(F, dtype=np.float64)
    C = np.ascontiguousarray(C, dtype=np.float64)
    A = np.zeros((2, 2))
    lib().orc_stress_affine_2d(_p(F), inv_dx, mu, lam, dt, vol, mass, _p(C), _p(A))
    return A
