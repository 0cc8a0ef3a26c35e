"""Host-side plumbing between PyTorch tensors and the C ABI of libfemflow_mpm.so.

PyTorch provides device memory and the current stream; every computation runs in the sm_103a
kernels.  Host (CPU / numpy) arrays are accepted by the reference-facing functions: they are
staged to the GPU through pinned buffers, computed there, and copied back in place.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N

_WS_CACHE: dict = {}


def _stream_ptr(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("femflow_gb300 needs a CUDA GPU (sm_103a); there is no CPU fallback")


def real_bytes(dtype) -> int:
    if dtype == torch.float32:
        return 4
    if dtype == torch.float64:
        return 8
    raise TypeError(f"unsupported dtype {dtype}: use float32 or float64")


def make_params(dim: int, res: int, dtype, dx: float, inv_dx: float, dt: float, gravity: float = 0.0,
                volume: float = 1.0, hardening: float = 1.0, mass: float = 0.0, mu_0: float = 0.0,
                lambda_0: float = 0.0, model="neo_hookean", wall_mode="reference", deterministic: bool = False,
                block_size: int = 0, variant: int = 0, planes=None, plane_rule="sticky", wait_limit: int = 0,
                inject: int = 0) -> N.Params:
    """Kernel parameters.  ``planes``: up to 8 planar colliders as (point, normal) pairs of ``dim``
    numbers each, applied by every grid update (``plane_rule`` "sticky" or "reference_literal",
    see ffmpm_params in include/femflow_mpm.h).  ``wait_limit`` bounds the sort's look-back wait
    (0: the library default) and ``inject`` takes N.INJECT_* bits; both are for tests of the
    bounded waits."""
    p = N.Params()
    p.dim, p.res, p.real_bytes = int(dim), int(res), real_bytes(dtype)
    p.model = N.MODELS[model] if isinstance(model, str) else int(model)
    p.wall_mode = N.WALLS[wall_mode] if isinstance(wall_mode, str) else int(wall_mode)
    p.deterministic, p.block_size, p.variant = int(bool(deterministic)), int(block_size), int(variant)
    p.dx, p.inv_dx, p.dt, p.gravity = float(dx), float(inv_dx), float(dt), float(gravity)
    p.volume, p.hardening = float(volume), float(hardening)
    p.mass, p.mu_0, p.lambda_0 = float(mass), float(mu_0), float(lambda_0)
    planes = list(planes or [])
    if len(planes) > N.MAX_PLANES:
        raise ValueError(f"at most {N.MAX_PLANES} planes")
    p.n_planes = len(planes)
    p.plane_rule = N.PLANE_RULES[plane_rule] if isinstance(plane_rule, str) else int(plane_rule)
    p.wait_limit, p.inject = int(wait_limit), int(inject)
    for q, (point, normal) in enumerate(planes):
        point, normal = np.asarray(point, dtype=np.float64), np.asarray(normal, dtype=np.float64)
        if point.shape != (dim,) or normal.shape != (dim,):
            raise ValueError(f"a plane is a point and a normal of {dim} numbers each")
        for d in range(dim):
            p.planes[q][d], p.planes[q][3 + d] = float(point[d]), float(normal[d])
    return p


def workspace_bytes(params: N.Params, n: int) -> int:
    out = ctypes.c_size_t(0)
    N.call("ffmpm_workspace_size", ctypes.byref(params), int(n), ctypes.byref(out))
    return int(out.value)


class Workspace:
    """Caller-owned scratch of the C ABI (torch allocation, 256-byte aligned), prepared once."""

    def __init__(self, params: N.Params, n: int, device):
        self.bytes = workspace_bytes(params, n)
        self.buf = torch.empty(self.bytes + 256, dtype=torch.uint8, device=device)
        base = self.buf.data_ptr()
        self.ptr = (base + 255) // 256 * 256
        self.device = device
        N.call("ffmpm_workspace_init", ctypes.byref(params), int(n), ctypes.c_void_p(self.ptr),
               ctypes.c_size_t(self.bytes), ctypes.c_void_p(_stream_ptr(device)))

    def status(self) -> tuple[int, int]:
        st, fb = ctypes.c_int32(0), ctypes.c_uint32(0)
        N.call("ffmpm_status_read", ctypes.c_void_p(self.ptr), ctypes.byref(st), ctypes.byref(fb),
               ctypes.c_void_p(_stream_ptr(self.device)))
        return int(st.value), int(fb.value)

    def clear_status(self):
        N.call("ffmpm_status_clear", ctypes.c_void_p(self.ptr), ctypes.c_void_p(_stream_ptr(self.device)))

    def raise_on_status(self):
        st, _ = self.status()
        if st:
            self.clear_status()
            raise RuntimeError(status_message(st))


def status_message(st: int) -> str:
    """What the FFMPM_STATUS_* bits of a status word report, most specific first."""
    parts = []
    if st & N.STATUS_OOB:
        parts.append("particle out of grid bounds (reference: RuntimeError in utils.oob)")
    if st & N.STATUS_NONFINITE:
        parts.append("non-finite value in the particle state (x, v, F or C)")
    if st & N.STATUS_TIMEOUT:
        parts.append("a bounded device wait expired; the results of the call are not valid")
    rest = st & ~(N.STATUS_OOB | N.STATUS_NONFINITE | N.STATUS_TIMEOUT)
    if rest or not parts:
        parts.append(f"device status {st:#x}")
    return "; ".join(parts)


def workspace_for(params: N.Params, n: int, device) -> Workspace:
    """Workspace cache keyed by the shape-determining parameters."""
    key = (params.dim, params.res, params.real_bytes, params.deterministic, params.block_size, int(n),
           torch.device(device).index)
    ws = _WS_CACHE.get(key)
    if ws is None:
        ws = Workspace(params, n, device)
        _WS_CACHE[key] = ws
    return ws


def ptr(t) -> int:
    return 0 if t is None else t.data_ptr()


def particles_struct(x, v, F, C, Jp, mass=None, mu_0=None, lambda_0=None, stride: int = 0, n: int | None = None
                     ) -> N.Particles:
    """Row-major arrays (stride 0) or component-major arrays of the given stride (then pass n)."""
    s = N.Particles()
    s.n = int(x.shape[0]) if n is None else int(n)
    s.stride = int(stride)
    s.x, s.v, s.F, s.C = ptr(x), ptr(v), ptr(F), ptr(C)
    s.Jp = ptr(Jp)
    s.mass, s.mu_0, s.lambda_0 = ptr(mass), ptr(mu_0), ptr(lambda_0)
    return s


def grid_struct(gv, gm) -> N.Grid:
    g = N.Grid()
    g.velocity, g.mass = ptr(gv), ptr(gm)
    return g


# ------------------------------------------------------------------------------- host staging
@dataclass
class Staged:
    """A set of arrays on the GPU, with the host originals they must be written back to."""

    dev: list
    host: list

    def write_back(self, indices):
        """Copy the device arrays back into their host originals; copies into pinned host tensors
        are queued together and waited for once."""
        pending = None
        for i in indices:
            h, d = self.host[i], self.dev[i]
            if h is None or d is None:
                continue
            if isinstance(h, np.ndarray):
                h[...] = d.cpu().numpy().astype(h.dtype, copy=False).reshape(h.shape)
            elif h is not d:
                pinned = h.is_pinned()
                h.copy_(d.view(h.shape), non_blocking=pinned)
                if pinned:
                    pending = d.device
        if pending is not None:
            torch.cuda.current_stream(pending).synchronize()


def stage(arrays, device=None, dtype=None) -> Staged:
    """Move host arrays (numpy or CPU tensors) to the GPU; CUDA tensors pass through."""
    _require_cuda()
    device = torch.device(device or "cuda")
    dev, host = [], []
    for a in arrays:
        if a is None:
            dev.append(None)
            host.append(None)
            continue
        if isinstance(a, np.ndarray):
            t = torch.from_numpy(np.ascontiguousarray(a))
            host.append(a)
        else:
            t = a
            host.append(a if not a.is_cuda else None)
        if t.is_cuda:
            if dtype is not None and t.dtype != dtype:
                raise TypeError(f"all arrays must share one dtype ({dtype}), got {t.dtype}")
            if not t.is_contiguous():
                raise TypeError("CUDA arrays are updated in place and must be contiguous")
        else:
            t = t.to(device, non_blocking=True)
            if dtype is not None and t.dtype != dtype:
                t = t.to(dtype)
        if not t.is_contiguous():
            t = t.contiguous()
        dev.append(t)
    return Staged(dev, host)


def check_tensors(dtype, *tensors):
    for t in tensors:
        if t is None:
            continue
        if not t.is_cuda:
            raise TypeError("tensor must be on a CUDA device")
        if t.dtype != dtype:
            raise TypeError(f"all arrays must share one dtype ({dtype}), got {t.dtype}")
        if not t.is_contiguous():
            raise TypeError("arrays must be contiguous")
