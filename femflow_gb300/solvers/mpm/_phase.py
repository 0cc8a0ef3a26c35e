"""Shared staging / call / write-back sequence of the reference-facing functions."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ... import _native as N
from ... import engine as E
from .particle import Particle, ParticleSet


def dtype_of(*arrays):
    for a in arrays:
        if a is None:
            continue
        if isinstance(a, np.ndarray):
            return torch.float64 if a.dtype == np.float64 else torch.float32
        if isinstance(a, torch.Tensor):
            return a.dtype
    return torch.float32


def split_particles(particles):
    """Returns (ParticleSet, list-or-None): a list of Particle objects is converted (host, float64)."""
    if isinstance(particles, ParticleSet):
        return particles, None
    if isinstance(particles, (list, tuple)) and (len(particles) == 0 or isinstance(particles[0], Particle)):
        return ParticleSet.from_particles(list(particles)), list(particles)
    raise TypeError("particles must be a ParticleSet or a list of Particle")


def stream(device) -> ctypes.c_void_p:
    return ctypes.c_void_p(E._stream_ptr(device))


def run(entry: str, params: N.Params, n: int, device, *args, check: bool = True):
    """Call a workspace-taking entry point, then raise like the reference on a device error."""
    ws = E.workspace_for(params, n, device)
    N.call(entry, *args, ctypes.c_void_p(ws.ptr), ctypes.c_size_t(ws.bytes), stream(device))
    if check:
        ws.raise_on_status()
    return ws
