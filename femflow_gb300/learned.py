"""Learned corrector: coarse MLS-MPM substeps (k times the fine dt) corrected by a per-particle MLP.

The plain method is the 3D substep of femflow/solvers/mpm/mls_mpm.py:40-79.  A coarse step runs
P2G and the grid update at dt_c = k dt (the C ABI's ffmpm_p2g / ffmpm_grid_op into a dense grid)
and then ``ffmpm_corrector_g2p``: the G2P fused with a 113 -> 64 -> 64 -> 64 -> 12 GELU network on
the tensor cores, which adds dF and dv to each particle's result.

* Data: fine-dt rollouts of seeded two-cube scenes generate the samples.  At a sample point the
  state is copied, one plain coarse step on the copy exports the features, and k fine steps on the
  original give the target (F_fine - F_coarse, (v_fine - v_coarse) dt_c / dx).
* Training: every GEMM of the forward and backward passes runs on the tcgen05 kernel
  (``ffmpm_mlp_train_*``), BF16 operands with FP32 accumulation, Adam on FP32 master weights.
* Rollout: every ``check_every`` coarse steps the range of det F and the total energy (FP64
  diagnostics) are checked; outside det F in [0.5, 2] or an energy gain above ``energy_tol`` the
  segment is discarded and redone with plain fine steps (the fallback).  The plain fine rollout is
  the yardstick: positions of the corrected and of the plain coarse rollouts are compared with it.
"""
from __future__ import annotations

import ctypes
import math
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from . import engine as E
from . import scenes
from .diff import pack

OUT_WEIGHTS = (1.0,) * 12


def _vp(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


class Net:
    """Corrector parameters and the training buffers of the tensor-core trainer (device memory)."""

    def __init__(self, device="cuda", max_batch: int = 65536, seed: int = 0):
        if max_batch % 128:
            raise ValueError("max_batch must be a multiple of 128")
        dev = torch.device(device)
        self.device, self.max_batch = dev, max_batch
        g = torch.Generator().manual_seed(seed)
        P = torch.zeros(N.MLP_PARAMS)

        def init(off, rows, cols, ld, gain):
            P[off:off + rows * ld].view(rows, ld)[:, :cols] = torch.randn(rows, cols, generator=g) * gain / math.sqrt(cols)

        init(N.MLP_OFF["W1"], 64, N.MLP_FEATURES, 128, math.sqrt(2.0))
        init(N.MLP_OFF["W2"], 64, 64, 64, math.sqrt(2.0))
        init(N.MLP_OFF["W3"], 64, 64, 64, math.sqrt(2.0))
        init(N.MLP_OFF["W4"], 12, 64, 64, 0.1)  # start close to "no correction"
        f32 = dict(dtype=torch.float32, device=dev)
        bf = dict(dtype=torch.bfloat16, device=dev)
        self.params = P.to(dev)
        self.grads = torch.zeros(N.MLP_PARAMS, **f32)
        self.adam_m = torch.zeros(N.MLP_PARAMS, **f32)
        self.adam_v = torch.zeros(N.MLP_PARAMS, **f32)
        self.W = {k: torch.zeros(s, **bf) for k, s in (("W1", (64, 128)), ("W2", (64, 64)), ("W3", (64, 64)),
                                                        ("W4", (16, 64)), ("W2t", (64, 64)), ("W3t", (64, 64)),
                                                        ("W4t", (64, 64)))}
        self.in_scale = torch.ones(N.MLP_IN, **f32)
        self.out_scale = torch.ones(16, **f32)
        B = max_batch
        self.buf = dict(Z1=torch.zeros(B, 64, **f32), Z2=torch.zeros(B, 64, **f32), Z3=torch.zeros(B, 64, **f32),
                        Y=torch.zeros(B, 16, **f32), dH=torch.zeros(B, 64, **f32),
                        H1=torch.zeros(B, 64, **bf), H2=torch.zeros(B, 64, **bf), H3=torch.zeros(B, 64, **bf),
                        H1t=torch.zeros(64, B, **bf), H2t=torch.zeros(64, B, **bf), H3t=torch.zeros(64, B, **bf),
                        Xt=torch.zeros(128, B, **bf), dY=torch.zeros(B, 64, **bf), dZ=torch.zeros(B, 64, **bf),
                        dYt=torch.zeros(128, B, **bf), dZt=torch.zeros(128, B, **bf))
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.step = 0
        self.repack()

    # -- C-ABI views
    def mlp(self, b4=None, out_scale=None) -> N.MLP:
        """C-ABI view; b4 / out_scale (device float[16]) override the trained output bias / scale."""
        m = N.MLP()
        m.W1, m.W2, m.W3, m.W4 = (self.W[k].data_ptr() for k in ("W1", "W2", "W3", "W4"))
        base, es = self.params.data_ptr(), 4
        m.b1, m.b2, m.b3, m.b4 = (base + es * N.MLP_OFF[k] for k in ("b1", "b2", "b3", "b4"))
        if b4 is not None:
            m.b4 = b4.data_ptr()
        m.in_scale = self.in_scale.data_ptr()
        m.out_scale = (self.out_scale if out_scale is None else out_scale).data_ptr()
        return m

    def trainer(self) -> N.MLPTrainer:
        t = N.MLPTrainer()
        t.max_batch = self.max_batch
        t.params, t.grads, t.adam_m, t.adam_v = (x.data_ptr() for x in (self.params, self.grads, self.adam_m,
                                                                          self.adam_v))
        for k in ("W1", "W2", "W3", "W4", "W2t", "W3t", "W4t"):
            setattr(t, k, self.W[k].data_ptr())
        for k, v in self.buf.items():
            setattr(t, k, v.data_ptr())
        t.status = self.status.data_ptr()
        return t

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def repack(self):
        """bf16 weights from the master parameters (an Adam step of rate 0 on zero gradients)."""
        self.grads.zero_()
        t = self.trainer()
        N.call("ffmpm_mlp_train_update", ctypes.byref(t), 0.0, 0.9, 0.999, 1e-8, 1, self._stream())

    # -- training primitives
    def forward_train(self, X: torch.Tensor) -> torch.Tensor:
        """Network output (before out_scale, with b4) for scaled bf16 features X [B][128]."""
        t = self.trainer()
        B = X.shape[0]
        N.call("ffmpm_mlp_train_forward", ctypes.byref(t), _vp(X), B, self._stream())
        return self.buf["Y"][:B, :12] + self.params[N.MLP_OFF["b4"]:N.MLP_OFF["b4"] + 12]

    def backward_train(self, T: torch.Tensor, w: torch.Tensor, loss: torch.Tensor):
        t = self.trainer()
        N.call("ffmpm_mlp_train_backward", ctypes.byref(t), _vp(T), _vp(w), T.shape[0], _vp(loss), self._stream())

    def update(self, lr: float, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step += 1
        t = self.trainer()
        N.call("ffmpm_mlp_train_update", ctypes.byref(t), float(lr), float(beta1), float(beta2), float(eps),
               self.step, self._stream())

    def check(self):
        if int(self.status.item()):
            raise RuntimeError("tensor-core wait timed out")

    # -- persistence
    def state(self) -> dict:
        return dict(params=self.params.cpu().numpy(), in_scale=self.in_scale.cpu().numpy(),
                    out_scale=self.out_scale.cpu().numpy())

    def load_state(self, st: dict):
        self.params.copy_(torch.as_tensor(st["params"]))
        self.in_scale.copy_(torch.as_tensor(st["in_scale"]))
        self.out_scale.copy_(torch.as_tensor(st["out_scale"]))
        self.repack()


class Corrector:
    """A trained network bound to one material: its output is taken relative to the network's output
    for the same material at rest (F = I, no motion), so that a body at rest or in rigid translation
    gets no correction, and scaled by `strength` (0 turns the network off)."""

    def __init__(self, net: Net, stepper: "Stepper", strength: float = 1.0):
        self.net = net
        raw = torch.zeros(N.MLP_IN, dtype=torch.float32, device=net.device)
        p = stepper.coarse
        kk = p.dt * p.dt * p.inv_dx * p.inv_dx * p.volume / p.mass
        raw[102], raw[103] = p.mu_0 * p.hardening * kk, p.lambda_0 * p.hardening * kk
        X = (raw * net.in_scale).to(torch.bfloat16).expand(128, N.MLP_IN).contiguous()
        f_rest = net.forward_train(X)[0]
        b4 = net.params[N.MLP_OFF["b4"]:N.MLP_OFF["b4"] + 16].clone()
        b4[:12] -= f_rest
        self.b4 = b4.contiguous()
        self.out_scale = (net.out_scale * strength).contiguous()
        self.strength = strength

    def mlp(self) -> N.MLP:
        return self.net.mlp(self.b4, self.out_scale)


@dataclass
class SceneSpec:
    n_per_cube: int = 131072
    edge: float = 0.2
    speed: float = 1.0
    E: float = 150.0
    nu: float = 0.3
    seed: int = 0


class Stepper:
    """Plain fine substeps and coarse (corrected or plain) substeps on a [24, n] float32 buffer."""

    def __init__(self, spec: SceneSpec, res: int = 128, dt: float = 5e-5, ratio: int = 8, gravity: float = -9.8,
                 model: str = "fixed_corotated", device="cuda"):
        s = scenes.two_cubes(spec.n_per_cube, spec.edge, spec.speed, spec.E, spec.nu, seed=spec.seed)
        self.scene, self.n, self.res, self.dt, self.ratio = s, s["n"], res, dt, ratio
        dev = torch.device(device)
        self.device = dev
        kw = dict(volume=s["vol"], hardening=1.0, mass=s["mass"], mu_0=s["mu"], lambda_0=s["lam"], model=model)
        self.fine = E.make_params(3, res, torch.float32, 1.0 / res, float(res), dt, gravity, **kw)
        self.coarse = E.make_params(3, res, torch.float32, 1.0 / res, float(res), dt * ratio, gravity, **kw)
        self.ws = E.workspace_for(self.fine, self.n, dev)
        R = res + 1
        self.gv = torch.zeros(R ** 3 * 3, dtype=torch.float32, device=dev)
        self.gm = torch.zeros(R ** 3, dtype=torch.float32, device=dev)
        self.Jp = torch.ones(self.n, dtype=torch.float32, device=dev)
        self.det = torch.zeros(2, dtype=torch.int32, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.diag = torch.zeros(8, dtype=torch.float64, device=dev)
        self.reset_det()

    def initial_state(self) -> torch.Tensor:
        f = dict(dtype=torch.float32, device=self.device)
        x = torch.as_tensor(self.scene["x"], **f)
        v = torch.as_tensor(self.scene["v"], **f)
        F = torch.eye(3, **f).expand(self.n, 3, 3)
        return pack(x, v, F, torch.zeros(self.n, 3, 3, **f))

    def _P(self, buf) -> N.Particles:
        P = N.Particles()
        P.n, P.stride = self.n, self.n
        base, es = buf.data_ptr(), 4
        P.x, P.v, P.F, P.C = (base + es * self.n * r for r in (0, 3, 6, 15))
        P.Jp = self.Jp.data_ptr()
        return P

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def fine_step(self, buf):
        P = self._P(buf)
        N.call("ffmpm_substep", ctypes.byref(self.fine), ctypes.byref(P), ctypes.c_void_p(self.ws.ptr),
               ctypes.c_size_t(self.ws.bytes), self._stream())

    def coarse_step(self, buf, net: "Corrector | Net | None" = None, features: torch.Tensor | None = None):
        P = self._P(buf)
        self.gv.zero_()
        self.gm.zero_()
        g = E.grid_struct(self.gv, self.gm)
        s = self._stream()
        N.call("ffmpm_p2g", ctypes.byref(self.coarse), ctypes.byref(P), ctypes.byref(g), ctypes.c_void_p(self.ws.ptr),
               ctypes.c_size_t(self.ws.bytes), s)
        N.call("ffmpm_grid_op", ctypes.byref(self.coarse), ctypes.byref(g), s)
        m = net.mlp() if net is not None else None
        N.call("ffmpm_corrector_g2p", ctypes.byref(self.coarse), ctypes.byref(g), ctypes.byref(P),
               ctypes.byref(m) if m is not None else None, _vp(features), _vp(self.det), _vp(self.status), s)

    def reset_det(self):
        self.det.copy_(torch.tensor([0x7FFFFFFF, -0x80000000], dtype=torch.int32))

    def det_range(self) -> tuple[float, float]:
        k = self.det.cpu().numpy().astype(np.int32)
        bits = np.where(k >= 0, k, k ^ np.int32(0x7FFFFFFF)).astype(np.int32)
        lo, hi = bits.view(np.float32)
        return float(lo), float(hi)

    def energy(self, buf) -> float:
        P = self._P(buf)
        N.call("ffmpm_diagnostics_fp64", ctypes.byref(self.fine), ctypes.byref(P), _vp(self.diag), self._stream())
        d = self.diag.cpu().tolist()
        return d[0] + d[1] + d[2]

    def check(self):
        self.ws.raise_on_status()
        if int(self.status.item()):
            st = int(self.status.item())
            self.status.zero_()
            raise RuntimeError(f"corrector G2P status {st:#x}")


def make_targets(st: Stepper, coarse_buf: torch.Tensor, fine_buf: torch.Tensor) -> torch.Tensor:
    """[n][12]: F_fine - F_coarse (9) and (v_fine - v_coarse) dt_c / dx (3)."""
    vs = st.dt * st.ratio * st.res
    dF = (fine_buf[6:15] - coarse_buf[6:15]).t()
    dv = (fine_buf[3:6] - coarse_buf[3:6]).t() * vs
    return torch.cat([dF, dv], dim=1).contiguous()


def _keep_rows(X, T, keep: float, gen: torch.Generator):
    """A random fraction `keep` of the rows of one sample (all rows for keep >= 1)."""
    if keep >= 1.0:
        return X, T
    m = max(1, int(X.shape[0] * keep))
    idx = torch.randperm(X.shape[0], generator=gen, device="cpu")[:m].to(X.device)
    return X[idx], T[idx]


def generate(specs, res=128, dt=5e-5, ratio=8, samples_per_scene=5, warm=40, gap=16, device="cuda", keep=1.0):
    """Features (bf16 [S][128], unscaled) and targets (float32 [S][12]) from fine rollouts; `keep`
    keeps a random fraction of each sample's particles (scenes as dense as the evaluated one without
    the full data volume)."""
    gen = torch.Generator().manual_seed(1234)
    feats, targs = [], []
    for spec in specs:
        st = Stepper(spec, res, dt, ratio, device=device)
        buf = st.initial_state()
        for _ in range(warm):
            st.fine_step(buf)
        for _ in range(samples_per_scene):
            tmp = buf.clone()
            X = torch.empty((st.n, N.MLP_IN), dtype=torch.bfloat16, device=st.device)
            st.coarse_step(tmp, None, X)
            for _ in range(ratio):
                st.fine_step(buf)
            Xk, Tk = _keep_rows(X, make_targets(st, tmp, buf), keep, gen)
            feats.append(Xk)
            targs.append(Tk)
            for _ in range(gap):
                st.fine_step(buf)
        st.check()
    return torch.cat(feats), torch.cat(targs)


def generate_on_policy(specs, cor_for, res=128, dt=5e-5, ratio=8, samples_per_scene=5, warm=5, gap=2,
                       device="cuda", keep=1.0):
    """Features and targets on the trajectory of the corrected coarse step itself: the state
    advances by corrected coarse steps (``cor_for(stepper)`` gives the Corrector), and at each sample
    point the target is the fine rollout of ``ratio`` substeps from that state against a plain coarse
    step from it.  Training on these states teaches the network the states it meets when it runs in
    closed loop, which fine rollouts alone do not show it.  A scene whose corrected trajectory
    leaves the grid contributes nothing (its status is cleared); the number of such scenes is
    returned third."""
    feats, targs, dropped = [], [], 0
    gen = torch.Generator().manual_seed(4321)
    for spec in specs:
        st = Stepper(spec, res, dt, ratio, device=device)
        cor = cor_for(st)
        buf = st.initial_state()
        f_scene, t_scene = [], []
        for _ in range(warm):
            st.coarse_step(buf, cor)
        for _ in range(samples_per_scene):
            tmp = buf.clone()
            X = torch.empty((st.n, N.MLP_IN), dtype=torch.bfloat16, device=st.device)
            st.coarse_step(tmp, None, X)
            fine = buf.clone()
            for _ in range(ratio):
                st.fine_step(fine)
            Xk, Tk = _keep_rows(X, make_targets(st, tmp, fine), keep, gen)
            f_scene.append(Xk)
            t_scene.append(Tk)
            for _ in range(1 + gap):
                st.coarse_step(buf, cor)
        if st.ws.status()[0] != 0 or int(st.status.item()) != 0:
            st.ws.clear_status()
            st.status.zero_()
            dropped += 1
            continue
        feats += f_scene
        targs += t_scene
    if not feats:
        return None, None, dropped
    return torch.cat(feats), torch.cat(targs), dropped


def training_specs(n_scenes: int, n_per_cube: int, seed: int = 0, E_range=(50.0, 200.0)):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_scenes):
        out.append(SceneSpec(n_per_cube=n_per_cube, E=float(np.exp(rng.uniform(*np.log(E_range)))),
                             nu=float(rng.uniform(0.2, 0.35)), speed=float(rng.uniform(0.5, 1.5)),
                             seed=int(seed * 1000 + i)))
    return out


def fit_scales(net: Net, X: torch.Tensor, T: torch.Tensor):
    """Input scale 1/std per feature (0 for constant ones), output scale std per target."""
    sd = X[:: max(1, X.shape[0] // 2_000_000)].float().std(dim=0)
    net.in_scale.copy_(torch.where(sd > 1e-12, 1.0 / sd, torch.zeros_like(sd)))
    so = T[:: max(1, T.shape[0] // 2_000_000)].std(dim=0)
    out = torch.ones(16, device=net.device)
    out[:12] = torch.where(so > 1e-20, so, torch.ones_like(so))
    net.out_scale.copy_(out)


def scaled(net: Net, X: torch.Tensor, T: torch.Tensor):
    Xs = (X.float() * net.in_scale).to(torch.bfloat16)
    Ts = (T / net.out_scale[:12]).contiguous()
    return Xs, Ts


def train(net: Net, Xs: torch.Tensor, Ts: torch.Tensor, steps: int = 3000, batch: int = 65536, lr: float = 2e-3,
          seed: int = 0, log_every: int = 100):
    """Adam with cosine decay on scaled features / targets; returns the logged training losses."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    perm = torch.randperm(Xs.shape[0], generator=g).to(Xs.device)
    Xs, Ts = Xs[perm].contiguous(), Ts[perm].contiguous()
    nb = Xs.shape[0] // batch
    w = torch.tensor(OUT_WEIGHTS, dtype=torch.float32, device=net.device)
    loss = torch.zeros(1, dtype=torch.float64, device=net.device)
    log = []
    for it in range(steps):
        b = it % nb
        X = Xs[b * batch:(b + 1) * batch]
        T = Ts[b * batch:(b + 1) * batch]
        net.forward_train(X)
        net.backward_train(T, w, loss)
        net.update(lr * 0.5 * (1 + math.cos(math.pi * it / steps)) + 1e-5)
        if (it + 1) % log_every == 0:
            log.append(float(loss.item()) / log_every)
            loss.zero_()
    net.check()
    return log


def evaluate_loss(net: Net, Xs: torch.Tensor, Ts: torch.Tensor, batch: int = 65536) -> float:
    """Mean weighted squared error of the network on (Xs, Ts); 1.0 ~ predicting zero correction."""
    tot, cnt = 0.0, 0
    for b in range(Xs.shape[0] // batch):
        Y = net.forward_train(Xs[b * batch:(b + 1) * batch])
        tot += float(((Y - Ts[b * batch:(b + 1) * batch]) ** 2).sum())
        cnt += batch
    return tot / max(cnt, 1)


def rollout_fine(st: Stepper, buf, n_fine: int):
    for _ in range(n_fine):
        st.fine_step(buf)


def rollout_coarse(st: Stepper, buf, n_coarse: int, net: "Corrector | Net | None" = None, check_every: int = 8,
                   det_bounds=(0.5, 2.0), energy_tol: float = 0.05) -> dict:
    """Coarse steps (corrected when `net` is given) with the det F / energy fallback to fine steps."""
    snap = buf.clone()
    e_prev = st.energy(buf)
    fallbacks, k = 0, 0
    while k < n_coarse:
        m = min(check_every, n_coarse - k)
        st.reset_det()
        for _ in range(m):
            st.coarse_step(buf, net)
        lo, hi = st.det_range()
        e = st.energy(buf)
        bad = not (det_bounds[0] <= lo and hi <= det_bounds[1]) or not math.isfinite(e) or \
            e > e_prev + energy_tol * abs(e_prev) or int(st.status.item()) != 0
        if bad:
            st.status.zero_()
            buf.copy_(snap)
            for _ in range(m * st.ratio):
                st.fine_step(buf)
            e = st.energy(buf)
            fallbacks += 1
        snap.copy_(buf)
        e_prev = e
        k += m
    return dict(fallback_segments=fallbacks, segments=math.ceil(n_coarse / check_every))


def position_error(buf, ref) -> dict:
    d = (buf[0:3] - ref[0:3]).abs()
    return dict(max=float(d.max()), mean=float(d.mean()))


def timed(fn, *a, **kw):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn(*a, **kw)
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0
