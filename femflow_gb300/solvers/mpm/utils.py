"""Scalar helpers of femflow/solvers/mpm/utils.py, for host-side setup code.

The per-particle versions of these formulas run inside the kernels (csrc/mpm_kernels.cuh).
"""
from __future__ import annotations

import math

import numpy as np


def constant_hardening(mu_0: float, lambda_0: float, e: float):
    """utils.py:7-24: (mu_0 * e, lambda_0 * e)."""
    return mu_0 * e, lambda_0 * e


def snow_hardening(mu_0: float, lambda_0: float, h: float, Jp: float):
    """utils.py:27-49: constant_hardening with e = exp(h * (1 - Jp))."""
    return constant_hardening(mu_0, lambda_0, math.exp(h * (1.0 - float(np.asarray(Jp).reshape(-1)[0]))))


def oob(base, res: int, ijk=(0, 0, 0)) -> bool:
    """utils.py:138-150: True if base + ijk leaves [0, res) on any axis."""
    tot = np.asarray(base) + np.asarray(ijk)
    return bool((tot >= res).any() or (tot < 0).any())


def Ev_to_mu(E: float, v: float) -> float:
    """femflow/numerics/fem.py:1-2."""
    return E / (2 * (1 + v))


def Ev_to_lambda(E: float, v: float) -> float:
    """femflow/numerics/fem.py:5-6."""
    return E * v / ((1 + v) * (1 - 2 * v))
