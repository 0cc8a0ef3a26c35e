"""Scene primitives of femflow/simulation/mpm/primitives.py, with the reference's conventions:

* ``grid(res)`` (femflow/numerics/geometry.py:100-116): lattice points in [0, 1]^d, first axis
  fastest, a unit axis mapped to 0.
* ``generate_implicit_points`` (primitives.py:46-61) keeps the lattice points whose implicit value,
  which already subtracts ``t``, is larger than ``t`` again (``inside > t``).  For the reference's
  three surfaces (by name, or this module's ``gyroid`` / ``diamond`` / ``primitive``) the lattice
  is evaluated and compacted on the GPU (``ffmpm_implicit_points``); a caller's own implicit
  function is Python code and is called point by point, as the reference calls it.
* ``primitive``, ``gyroid``, ``diamond`` (primitives.py:9-38) also take arrays of points [..., 3].
* ``generate_cube_points`` (primitives.py:64-76) emits each point as (z, y, x) with x fastest.
"""
from __future__ import annotations

import ctypes
from typing import Callable, Tuple, Union

import numpy as np
import torch

from ... import _native as N
from ... import engine as E


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


_KINDS = {"gyroid": 0, "diamond": 1, "primitive": 2}
_NAMES = {gyroid: "gyroid", diamond: "diamond", primitive: "primitive"}


def implicit_points_gpu(name: str, k: float, t: float, res: int, device="cuda") -> torch.Tensor:
    """The kept lattice points of one of the reference's surfaces, [m, 3] float64 on ``device``."""
    E._require_cuda()
    if name not in _KINDS:
        raise ValueError("Invalid implicit function specified")
    device = torch.device(device)
    nbytes = ctypes.c_size_t(0)
    N.call("ffmpm_implicit_points_workspace_size", int(res), ctypes.byref(nbytes))
    ws = torch.empty(int(nbytes.value), dtype=torch.uint8, device=device)
    count = torch.zeros(1, dtype=torch.int64, device=device)
    stream = ctypes.c_void_p(E._stream_ptr(device))
    args = (_KINDS[name], float(k), float(t), int(res))
    # first pass sizes the output, second pass writes it
    N.call("ffmpm_implicit_points", *args, None, 0, ctypes.c_void_p(count.data_ptr()), ctypes.c_void_p(ws.data_ptr()),
           nbytes, stream)
    m = int(count.item())
    out = torch.empty((m, 3), dtype=torch.float64, device=device)
    if m:
        N.call("ffmpm_implicit_points", *args, ctypes.c_void_p(out.data_ptr()), m, ctypes.c_void_p(count.data_ptr()),
               ctypes.c_void_p(ws.data_ptr()), nbytes, stream)
    return out


def generate_implicit_points(implicit_fn: Union[Callable, str], k: float, t: float, res: int) -> np.ndarray:
    if isinstance(implicit_fn, str):
        if implicit_fn not in _KINDS:
            raise ValueError("Invalid implicit function specified")
        name = implicit_fn
    else:
        name = _NAMES.get(implicit_fn)
    if name is not None:
        return implicit_points_gpu(name, k, t, res).cpu().numpy()
    g = grid((res, res, res))
    inside = np.array([implicit_fn(k, t, row) for row in g])
    return g[inside > t]


def generate_cube_points(xb: Tuple[float, float], yb: Tuple[float, float], zb: Tuple[float, float],
                         res: int = 10) -> np.ndarray:
    x = np.linspace(*xb, num=res)
    y = np.linspace(*yb, num=res)
    z = np.linspace(*zb, num=res)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return np.stack([Z.reshape(-1), Y.reshape(-1), X.reshape(-1)], axis=1).astype(np.float64)
