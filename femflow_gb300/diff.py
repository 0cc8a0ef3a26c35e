"""Differentiable 3D and 2D MLS-MPM rollouts with a hand-written adjoint.

``simulate(x0, v0, mu_0, lambda_0, cfg)`` runs ``cfg.steps`` substeps of the 3D solver
(``solve_mls_mpm_3d``, femflow/solvers/mpm/mls_mpm.py:40-79) or, for [n, 2] states, of the 2D
substep (femflow/solvers/mpm/two_d/*.py); model "neo_hookean" as the reference, or the textbook
"fixed_corotated" stress.  It runs on the GPU and
returns the final x, v, F, C as tensors that carry gradients back to x0, v0, F0, C0 and the
per-particle Lamé parameters.  Backward is the reverse-mode sweep of ``ffmpm_substep_adjoint``:

* the forward keeps a checkpoint of the particle state every ``cfg.checkpoint_every`` substeps;
* backward walks the segments last to first: it re-runs a segment's substeps from its checkpoint,
  keeping each intermediate state, then applies the adjoint substeps in reverse order.

Memory is ``steps / K`` checkpoints plus ``K`` states of one segment (24 reals per particle each
in 3D, 12 in 2D); compute is two forward passes plus one adjoint pass.  The state is held
component-major ([24, n]: x 0-2, v 3-5, F 6-14, C 15-23; 2D [12, n]: x 0-1, v 2-3, F 4-7,
C 8-11) so every kernel access is coalesced.

Gradients with respect to Young's modulus and Poisson's ratio follow by autograd through
``lame(E, nu)`` (femflow/numerics/fem.py:1-6), written with torch ops.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from . import _native as N
from . import engine as E

@dataclass(frozen=True)
class RolloutConfig:
    res: int
    dt: float
    steps: int
    volume: float
    checkpoint_every: int = 50
    gravity: float = -9.8
    hardening: float = 1.0
    wall_mode: str = "reference"
    # "neo_hookean": the reference's stress (lam(J-1)J on all nine entries of PF, utils.py:129);
    # "fixed_corotated": the textbook fixed-corotated stress (lam(J-1)J on the diagonal only)
    model: str = "neo_hookean"
    # planar colliders ((point, normal) pairs) applied by every grid update, and their rule
    planes: tuple = ()
    plane_rule: str = "sticky"


def lame(E_mod, nu):
    """(mu, lambda) of Young's modulus and Poisson's ratio, differentiable (numerics/fem.py:1-6)."""
    return E_mod / (2 * (1 + nu)), E_mod * nu / ((1 + nu) * (1 - 2 * nu))


def _rows(dim: int):
    """Row offsets of x, v, F, C in the component-major buffer, and its row count."""
    return (0, dim, 2 * dim, 2 * dim + dim * dim), 2 * dim + 2 * dim * dim


def pack(x, v, F, C) -> torch.Tensor:
    """Row-major x[n,d], v[n,d], F[n,d,d], C[n,d,d] -> one component-major [2d + 2d^2, n] buffer."""
    n, d = x.shape[0], x.shape[-1]
    return torch.cat([x.reshape(n, d).t(), v.reshape(n, d).t(), F.reshape(n, d * d).t(), C.reshape(n, d * d).t()],
                     dim=0).contiguous()


def unpack(buf: torch.Tensor):
    n = buf.shape[1]
    d = 3 if buf.shape[0] == 24 else 2
    (ox, ov, oF, oC), rows = _rows(d)
    x = buf[ox:ov].t().contiguous()
    v = buf[ov:oF].t().contiguous()
    F = buf[oF:oC].t().contiguous().reshape(n, d, d)
    C = buf[oC:rows].t().contiguous().reshape(n, d, d)
    return x, v, F, C


class _Runner:
    """The C-ABI calls of one rollout: forward substeps and adjoint substeps on [24, n] buffers."""

    def __init__(self, cfg: RolloutConfig, n: int, dtype, device, mass, mu_0, lambda_0, dim: int = 3):
        self.n = n
        self.dim = dim
        self.dtype = dtype
        self.device = device
        self.params = E.make_params(dim, cfg.res, dtype, 1.0 / cfg.res, float(cfg.res), cfg.dt, cfg.gravity,
                                    cfg.volume, cfg.hardening, model=cfg.model, wall_mode=cfg.wall_mode,
                                    planes=cfg.planes, plane_rule=cfg.plane_rule)
        if torch.is_tensor(mass):
            self.mass = mass.detach().to(device=device, dtype=dtype).reshape(n).contiguous()
        else:
            self.mass = None
            self.params.mass = float(mass)
        self.mu = mu_0.detach().to(device=device, dtype=dtype).reshape(n).contiguous()
        self.lam = lambda_0.detach().to(device=device, dtype=dtype).reshape(n).contiguous()
        self.Jp = torch.ones(n, dtype=dtype, device=device)
        self.ws = E.workspace_for(self.params, n, device)
        self.adj_bytes = ctypes.c_size_t(0)
        N.call("ffmpm_adjoint_workspace_size", ctypes.byref(self.params), n, ctypes.byref(self.adj_bytes))
        self.adj_buf = torch.zeros(self.adj_bytes.value + 256, dtype=torch.uint8, device=device)
        self.adj_ptr = (self.adj_buf.data_ptr() + 255) // 256 * 256
        self.stream = ctypes.c_void_p(E._stream_ptr(device))

    def _particles(self, buf: torch.Tensor) -> N.Particles:
        P = N.Particles()
        P.n, P.stride = self.n, self.n
        base, es = buf.data_ptr(), buf.element_size()
        P.x, P.v, P.F, P.C = (base + es * self.n * r0 for r0 in _rows(self.dim)[0])
        P.Jp = self.Jp.data_ptr()
        P.mass = self.mass.data_ptr() if self.mass is not None else None
        P.mu_0, P.lambda_0 = self.mu.data_ptr(), self.lam.data_ptr()
        return P

    def substep(self, buf: torch.Tensor):
        P = self._particles(buf)
        N.call("ffmpm_substep", ctypes.byref(self.params), ctypes.byref(P), ctypes.c_void_p(self.ws.ptr),
               ctypes.c_size_t(self.ws.bytes), self.stream)

    def adjoint(self, state: torch.Tensor, adj: torch.Tensor, mu_bar: torch.Tensor, lam_bar: torch.Tensor):
        P = self._particles(state)
        A = N.Adjoint()
        base, es = adj.data_ptr(), adj.element_size()
        A.x, A.v, A.F, A.C = (base + es * self.n * r0 for r0 in _rows(self.dim)[0])
        A.mu_0, A.lambda_0 = mu_bar.data_ptr(), lam_bar.data_ptr()
        N.call("ffmpm_substep_adjoint", ctypes.byref(self.params), ctypes.byref(P), ctypes.byref(A),
               ctypes.c_void_p(self.adj_ptr), ctypes.c_size_t(self.adj_bytes.value), self.stream)

    def check(self):
        self.ws.raise_on_status()
        st, fb = ctypes.c_int32(0), ctypes.c_uint32(0)
        N.call("ffmpm_status_read", ctypes.c_void_p(self.adj_ptr), ctypes.byref(st), ctypes.byref(fb), self.stream)
        if st.value:
            N.call("ffmpm_status_clear", ctypes.c_void_p(self.adj_ptr), self.stream)
            raise RuntimeError(f"adjoint substep: device status {st.value:#x} (1 = particle out of grid bounds)")


class MPMRollout(torch.autograd.Function):
    """x0, v0, F0, C0, mu_0, lambda_0 -> x, v, F, C after cfg.steps substeps.

    mu_0 / lambda_0 are [n] (per particle) or 0-dim (one material).  Their gradients are accumulated
    per particle in float64; for a 0-dim parameter the sum over particles is also taken in float64
    and rounded once (the per-particle terms nearly cancel: a float32 sum of float32 terms loses
    about 1e-2 of the total at 1e5 particles)."""

    @staticmethod
    def forward(ctx, x0, v0, F0, C0, mu_0, lambda_0, mass, cfg: RolloutConfig):
        n = x0.shape[0]
        ctx.scalar_mu, ctx.scalar_lam = mu_0.dim() == 0, lambda_0.dim() == 0
        runner = _Runner(cfg, n, x0.dtype, x0.device, mass, mu_0.expand(n), lambda_0.expand(n), dim=x0.shape[1])
        buf = pack(x0.detach(), v0.detach(), F0.detach(), C0.detach())
        K = max(1, int(cfg.checkpoint_every))
        ckpts = []
        for s in range(cfg.steps):
            if s % K == 0:
                ckpts.append(buf.clone())
            runner.substep(buf)
        runner.check()
        ctx.runner, ctx.ckpts, ctx.cfg = runner, ckpts, cfg
        return unpack(buf)

    @staticmethod
    def backward(ctx, gx, gv, gF, gC):
        runner, ckpts, cfg = ctx.runner, ctx.ckpts, ctx.cfg
        n, dtype, dev = runner.n, runner.dtype, runner.device

        def z(g, shape):
            return torch.zeros(shape, dtype=dtype, device=dev) if g is None else g.to(dtype)

        d = runner.dim
        adj = pack(z(gx, (n, d)), z(gv, (n, d)), z(gF, (n, d, d)), z(gC, (n, d, d)))
        mu_bar = torch.zeros(n, dtype=torch.float64, device=dev)
        lam_bar = torch.zeros(n, dtype=torch.float64, device=dev)
        K = max(1, int(cfg.checkpoint_every))
        seg = torch.empty((min(K, cfg.steps), _rows(d)[1], n), dtype=dtype, device=dev)
        for si in reversed(range(len(ckpts))):
            count = min(K, cfg.steps - si * K)
            seg[0].copy_(ckpts[si])
            for k in range(1, count):
                seg[k].copy_(seg[k - 1])
                runner.substep(seg[k])
            for k in reversed(range(count)):
                runner.adjoint(seg[k], adj, mu_bar, lam_bar)
        runner.check()
        gx0, gv0, gF0, gC0 = unpack(adj)
        ctx.runner = ctx.ckpts = None
        g_mu = mu_bar.sum() if ctx.scalar_mu else mu_bar
        g_lam = lam_bar.sum() if ctx.scalar_lam else lam_bar
        return gx0, gv0, gF0, gC0, g_mu.to(dtype), g_lam.to(dtype), None, None


def cell_order(x: torch.Tensor, res: int) -> torch.Tensor:
    """Stable order of particles by base cell (the node a particle's stencil starts at)."""
    R = res + 1
    b = torch.clamp(torch.floor(x.detach() * res - 0.5), -1, res).to(torch.int64) + 1
    key = b[:, 0]
    for a in range(1, x.shape[1]):
        key = key * (R + 2) + b[:, a]
    return torch.argsort(key, stable=True)


def simulate(x0, v0, mu_0, lambda_0, cfg: RolloutConfig, mass, F0=None, C0=None, order: bool = True):
    """Differentiable rollout of cfg.steps substeps; returns (x, v, F, C) at the end.

    x0, v0: [n, 3] (3D) or [n, 2] (2D) CUDA tensors (float32 or float64); mu_0, lambda_0: scalars / 0-dim tensors (one
    material) or [n] tensors (autograd-tracked, e.g. from ``lame(E, nu)``); mass: float or [n]
    tensor (not differentiated).
    F0, C0 default to the reference's initial state (identity, zero; mls_mpm.py:9-15).
    With ``order`` the rollout runs on the particles ordered by base cell (neighbouring lanes of the
    adjoint kernels then share stencil nodes); inputs and outputs stay in the caller's order, and
    autograd carries the permutation.
    """
    n, d = x0.shape[0], x0.shape[1]
    dtype, dev = x0.dtype, x0.device
    if F0 is None:
        F0 = torch.eye(d, dtype=dtype, device=dev).expand(n, d, d)
    if C0 is None:
        C0 = torch.zeros((n, d, d), dtype=dtype, device=dev)
    mu = torch.as_tensor(mu_0, dtype=dtype, device=dev)
    lam = torch.as_tensor(lambda_0, dtype=dtype, device=dev)
    if not order or n < 2:
        return MPMRollout.apply(x0, v0, F0, C0, mu, lam, mass, cfg)
    perm = cell_order(x0, cfg.res)
    inv = torch.empty_like(perm)
    inv[perm] = torch.arange(n, device=perm.device)
    pick = lambda t: t[perm] if torch.is_tensor(t) and t.dim() >= 1 and t.shape[0] == n else t
    out = MPMRollout.apply(pick(x0), pick(v0), pick(F0), pick(C0), pick(mu), pick(lam), pick(mass), cfg)
    return tuple(o[inv] for o in out)
