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


def pinned_host(*arrays) -> bool:
    """True when every array is a contiguous CPU tensor in page-locked memory, all of one float
    dtype: the arrays the pipelined host substep can copy while its kernels run."""
    ts = [a for a in arrays if a is not None]
    return bool(ts) and all(isinstance(a, torch.Tensor) and not a.is_cuda and a.is_pinned() and a.is_contiguous()
                            and a.dtype == ts[0].dtype for a in ts) and ts[0].dtype in (torch.float32, torch.float64)


_MIRRORS: dict = {}


def _device_mirror(arrays, device):
    """Device tensors shaped like the host arrays (kept between calls of the same shapes)."""
    key = (tuple(None if a is None else tuple(a.shape) for a in arrays), arrays[0].dtype, str(device))
    m = _MIRRORS.get(key)
    if m is None:
        m = [None if a is None else torch.empty(a.shape, dtype=a.dtype, device=device) for a in arrays]
        _MIRRORS[key] = m
    return m


def run_host_substep(params: N.Params, x, mass, mu_0, lambda_0, v, F, C, Jp, check: bool = True, device=None):
    """One substep on pinned host arrays through ffmpm_substep_host (copies pipelined with the
    kernels), in place; returns once the host arrays hold the result."""
    device = torch.device(device or "cuda")
    host = E.particles_struct(x, v, F, C, Jp, mass, mu_0, lambda_0)
    dx, dv, dF, dC, dJ, dm, dmu, dlam = _device_mirror([x, v, F, C, Jp, mass, mu_0, lambda_0], device)
    dev = E.particles_struct(dx, dv, dF, dC, dJ, dm, dmu, dlam)
    ws = E.workspace_for(params, host.n, device)
    N.call("ffmpm_substep_host", ctypes.byref(params), ctypes.byref(host), ctypes.byref(dev), ctypes.c_void_p(ws.ptr),
           ctypes.c_size_t(ws.bytes), stream(device))
    if check:
        ws.raise_on_status()  # synchronises the stream
    else:
        torch.cuda.current_stream(device).synchronize()


def run(entry: str, params: N.Params, n: int, device, *args, check: bool = True):
    """Call a workspace-taking entry point, then raise like the reference on a device error."""
    ws = E.workspace_for(params, n, device)
    N.call(entry, *args, ctypes.c_void_p(ws.ptr), ctypes.c_size_t(ws.bytes), stream(device))
    if check:
        ws.raise_on_status()
    return ws
