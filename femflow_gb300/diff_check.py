"""Gradient check of differentiable 3D rollouts against FP64 central finite differences.

Scene: a seeded-uniform cube (edge 0.25, centre (0.5, 0.5, 0.5)) with per-particle initial
velocities v0 ~ N(0, 0.1^2), fixed-corotated material from (E, nu), rho = 1, gravity -9.8,
particle volume = cube volume / n.  The material model defaults to the textbook fixed-corotated
stress: with the reference's stress (lam(J-1)J on all nine entries of PF) a free-falling elastic
cube at this resolution and step grows without bound over 2000 substeps for any E >= 1e3.
Two losses of the final positions:

* ``com``:    |centre of mass - (0.7, 0.3, 0.5)|^2 (the loss of the differentiable configuration)
* ``spread``: mean_p |x_p - centre of mass|^2 (depends on the material only weakly: E dL/dE / L is
  about 1e-4, so float32 rounding along the trajectory moves its float32 E-derivative by ~1e-2)
* ``strain``: mean_p |F_p - I|^2 of the final deformation gradients (depends on E and nu at order 1)

Gradients with respect to v0 (directional, along a seeded random direction), E and nu come from
the hand-written adjoint in float32 and in float64 and are compared with FP64 central
differences of the forward rollout.  Grid momentum is conserved away from the walls, so the
centre of mass moves as a free body: d(com loss)/d v0_p = 2 (com - target) T m_p / M, and its
E and nu derivatives vanish; both are checked as well.

    python -m femflow_gb300.diff_check --n 131072 --res 64 --steps 2000 --every 50
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from .diff import RolloutConfig, lame, simulate

TARGET = (0.7, 0.3, 0.5)


def cube_scene(n: int, edge: float = 0.25, centre=(0.5, 0.5, 0.5), vstd: float = 0.1, seed: int = 0,
               f0_std: float = 0.0):
    """Positions, initial velocities, a probe direction for v0, particle volume and the initial
    deformation gradient (identity, or identity plus N(0, f0_std^2) entries: a pre-strained body)."""
    rng = np.random.default_rng(seed)
    x0 = rng.uniform(-edge / 2, edge / 2, (n, 3)) + np.asarray(centre)
    v0 = rng.normal(0.0, vstd, (n, 3))
    direction = rng.normal(0.0, 1.0, (n, 3))
    vol = edge ** 3 / n
    F0 = np.eye(3)[None] + (rng.normal(0.0, f0_std, (n, 3, 3)) if f0_std > 0 else np.zeros((n, 3, 3)))
    return x0, v0, direction, vol, F0


LOSSES = ("com", "spread", "strain")


def losses(x: torch.Tensor, F: torch.Tensor):
    x, F = x.double(), F.double()
    com = x.mean(dim=0)
    t = torch.tensor(TARGET, dtype=torch.float64, device=x.device)
    eye = torch.eye(3, dtype=torch.float64, device=x.device)
    return {"com": ((com - t) ** 2).sum(), "spread": ((x - com) ** 2).sum(dim=1).mean(),
            "strain": ((F - eye) ** 2).sum(dim=(1, 2)).mean()}


def _rollout(x0, v0, E_mod, nu, cfg, mass, dtype, dev, F0):
    mu, lam = lame(E_mod, nu)
    x = torch.as_tensor(x0, dtype=dtype, device=dev)
    F = torch.as_tensor(F0, dtype=dtype, device=dev)
    return simulate(x, v0, mu.to(dtype), lam.to(dtype), cfg, mass, F0=F)


def adjoint_grads(x0, v0, direction, E_mod, nu, cfg, mass, dtype, dev, loss_name, F0):
    """Loss value and its derivatives (v0 along `direction`, full v0, E, nu) by the adjoint."""
    v = torch.as_tensor(v0, dtype=dtype, device=dev).clone().requires_grad_(True)
    Et = torch.tensor(E_mod, dtype=torch.float64, device=dev, requires_grad=True)
    nt = torch.tensor(nu, dtype=torch.float64, device=dev, requires_grad=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xT, vT, FT, CT = _rollout(x0, v, Et, nt, cfg, mass, dtype, dev, F0)
    L = losses(xT, FT)[loss_name]
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    L.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    d = torch.as_tensor(direction, dtype=torch.float64, device=dev)
    return dict(loss=float(L.detach()), dv=float((v.grad.double() * d).sum()), gv=v.grad.double(), dE=float(Et.grad),
                dnu=float(nt.grad), forward_s=t1 - t0, backward_s=t2 - t1)


def fd_loss(x0, v0, E_mod, nu, cfg, mass, dev, F0):
    with torch.no_grad():
        v = torch.as_tensor(v0, dtype=torch.float64, device=dev)
        xT, vT, FT, CT = _rollout(x0, v, torch.tensor(E_mod, dtype=torch.float64, device=dev),
                                  torch.tensor(nu, dtype=torch.float64, device=dev), cfg, mass, torch.float64, dev, F0)
        return {k: float(val) for k, val in losses(xT, FT).items()}


def central_differences(x0, v0, direction, E_mod, nu, cfg, mass, dev, F0, eps_v=1e-4, rel_E=1e-4, eps_nu=1e-4):
    """FP64 central differences of every loss along v0-direction, E and nu."""
    out = {}
    lp = fd_loss(x0, v0 + eps_v * direction, E_mod, nu, cfg, mass, dev, F0)
    lm = fd_loss(x0, v0 - eps_v * direction, E_mod, nu, cfg, mass, dev, F0)
    out["dv"] = {k: (lp[k] - lm[k]) / (2 * eps_v) for k in lp}
    h = rel_E * E_mod
    lp = fd_loss(x0, v0, E_mod + h, nu, cfg, mass, dev, F0)
    lm = fd_loss(x0, v0, E_mod - h, nu, cfg, mass, dev, F0)
    out["dE"] = {k: (lp[k] - lm[k]) / (2 * h) for k in lp}
    lp = fd_loss(x0, v0, E_mod, nu + eps_nu, cfg, mass, dev, F0)
    lm = fd_loss(x0, v0, E_mod, nu - eps_nu, cfg, mass, dev, F0)
    out["dnu"] = {k: (lp[k] - lm[k]) / (2 * eps_nu) for k in lp}
    return out


def adjoint_along(x0, v0, E_mod, nu, cfg, mass, dev, F0, fwd_dtype, adj_dtype, loss_name):
    """(dL/dE, dL/dnu) from the adjoint in `adj_dtype` applied along the forward trajectory of
    `fwd_dtype` (checkpoints and recomputed states rounded to adj_dtype).  A float32 adjoint along
    the float64 trajectory separates the adjoint's own arithmetic from the float32 trajectory."""
    from . import diff as Dm
    n = x0.shape[0]
    mu, lam = (float(a) for a in lame(E_mod, nu))
    run = {dt: Dm._Runner(cfg, n, dt, dev, mass, torch.full((n,), mu, dtype=torch.float64),
                          torch.full((n,), lam, dtype=torch.float64)) for dt in {fwd_dtype, adj_dtype}}

    def t(a, dt):
        return torch.as_tensor(a, dtype=dt, device=dev)

    buf = Dm.pack(t(x0, fwd_dtype), t(v0, fwd_dtype), t(F0, fwd_dtype), torch.zeros((n, 3, 3), dtype=fwd_dtype,
                                                                                        device=dev))
    K = max(1, int(cfg.checkpoint_every))
    ck = []
    for s in range(cfg.steps):
        if s % K == 0:
            ck.append(buf.clone())
        run[fwd_dtype].substep(buf)
    xT, vT, FT, CT = Dm.unpack(buf)
    xT = xT.double().requires_grad_(True)
    FT = FT.double().requires_grad_(True)
    gx, gF = torch.autograd.grad(losses(xT, FT)[loss_name], (xT, FT), allow_unused=True)
    gx = torch.zeros_like(xT) if gx is None else gx
    gF = torch.zeros_like(FT) if gF is None else gF
    adj = Dm.pack(gx, torch.zeros_like(gx), gF, torch.zeros_like(gF)).to(adj_dtype)
    mub = torch.zeros(n, dtype=torch.float64, device=dev)
    lamb = torch.zeros_like(mub)
    seg = torch.empty((min(K, cfg.steps), 24, n), dtype=fwd_dtype, device=dev)
    for si in reversed(range(len(ck))):
        count = min(K, cfg.steps - si * K)
        seg[0].copy_(ck[si])
        for k in range(1, count):
            seg[k].copy_(seg[k - 1])
            run[fwd_dtype].substep(seg[k])
        for k in reversed(range(count)):
            run[adj_dtype].adjoint(seg[k].to(adj_dtype).contiguous(), adj, mub, lamb)
    for r in run.values():
        r.check()
    a, b = float(mub.sum()), float(lamb.sum())
    # mu = E / (2 (1 + nu)), lam = E nu / ((1 + nu)(1 - 2 nu))
    dE = a / (2 * (1 + nu)) + b * nu / ((1 + nu) * (1 - 2 * nu))
    dnu = -a * E_mod / (2 * (1 + nu) ** 2) + b * E_mod * (1 + 2 * nu * nu) / ((1 + nu) ** 2 * (1 - 2 * nu) ** 2)
    return dE, dnu


def rel(a: float, b: float) -> float:
    return abs(a - b) / max(abs(b), 1e-300)


def run(n=131072, res=64, steps=2000, every=50, dt=1e-4, E_mod=4e3, nu=0.3, seed=0, model="fixed_corotated",
        f0_std=0.0, device="cuda") -> dict:
    dev = torch.device(device)
    x0, v0, direction, vol, F0 = cube_scene(n, seed=seed, f0_std=f0_std)
    mass = 1.0 * vol
    cfg = RolloutConfig(res=res, dt=dt, steps=steps, volume=vol, checkpoint_every=every, model=model)
    report = dict(n=n, res=res, steps=steps, checkpoint_every=every, dt=dt, E=E_mod, nu=nu, seed=seed, model=model,
                  f0_std=f0_std)
    t0 = time.perf_counter()
    fd = central_differences(x0, v0, direction, E_mod, nu, cfg, mass, dev, F0)
    report["fd_seconds"] = time.perf_counter() - t0
    for name in LOSSES:
        res_l = {}
        for dtype in (torch.float32, torch.float64):
            g = adjoint_grads(x0, v0, direction, E_mod, nu, cfg, mass, dtype, dev, name, F0)
            tag = "fp32" if dtype == torch.float32 else "fp64"
            gv = g.pop("gv")
            res_l[tag] = g
            res_l[tag + "_gv"] = gv
        g32, g64 = res_l["fp32"], res_l["fp64"]
        entry = {"fp32": g32, "fp64": g64,
                 "fd": {"dv": fd["dv"][name], "dE": fd["dE"][name], "dnu": fd["dnu"][name]}}
        for k in ("dv", "dE", "dnu"):
            entry[f"rel_fp32_vs_fd_{k}"] = rel(g32[k], fd[k][name])
            entry[f"rel_fp64_vs_fd_{k}"] = rel(g64[k], fd[k][name])
        a, b = res_l["fp32_gv"], res_l["fp64_gv"]
        entry["rel_fp32_vs_fp64_gv"] = float((a - b).norm() / b.norm())
        if name != "com":
            dE_m, dnu_m = adjoint_along(x0, v0, E_mod, nu, cfg, mass, dev, F0, torch.float64, torch.float32, name)
            entry["fp32_adjoint_on_fp64_trajectory"] = {"dE": dE_m, "dnu": dnu_m}
            entry["rel_fp32_adjoint_on_fp64_trajectory_vs_fd_dE"] = rel(dE_m, fd["dE"][name])
            entry["rel_fp32_adjoint_on_fp64_trajectory_vs_fd_dnu"] = rel(dnu_m, fd["dnu"][name])
        if name == "com":
            # free-body centre of mass: dL/dv0_p = 2 (com - target) T m_p / M (uniform mass: T / n)
            with torch.no_grad():
                xT, *_ = _rollout(x0, torch.as_tensor(v0, dtype=torch.float64, device=dev),
                                  torch.tensor(E_mod, dtype=torch.float64, device=dev),
                                  torch.tensor(nu, dtype=torch.float64, device=dev), cfg, mass, torch.float64, dev,
                                  F0)
                com = xT.mean(dim=0)
                t = torch.tensor(TARGET, dtype=torch.float64, device=dev)
                closed = (2 * (com - t) * (steps * dt) / n).expand(n, 3)
            entry["rel_fp32_vs_closed_form_gv"] = float((a - closed).norm() / closed.norm())
            entry["rel_fp64_vs_closed_form_gv"] = float((b - closed).norm() / closed.norm())
            # scale of the E / nu derivatives against the loss: these vanish for a free body
            entry["E_dE_over_loss_fp32"] = abs(g32["dE"] * E_mod) / g32["loss"]
        report[name] = entry
    return report


def time_backward(n=131072, res=64, steps=400, every=50, dt=1e-4, E_mod=4e3, nu=0.3, seed=0,
                  model="fixed_corotated", reps=2, device="cuda") -> dict:
    """Wall time of the float32 forward and backward of the spread loss over `steps` substeps of the
    cube scene (CUDA-synchronised), best of `reps`; no finite differences."""
    dev = torch.device(device)
    x0, v0, direction, vol, F0 = cube_scene(n, seed=seed)
    cfg = RolloutConfig(res=res, dt=dt, steps=steps, volume=vol, checkpoint_every=every, model=model)
    best = None
    for _ in range(reps):
        E = torch.tensor(E_mod, dtype=torch.float64, device=dev, requires_grad=True)
        nuv = torch.tensor(nu, dtype=torch.float64, device=dev, requires_grad=True)
        v = torch.as_tensor(v0, dtype=torch.float32, device=dev).requires_grad_(True)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        xs, _, Fs, _ = _rollout(x0, v, E, nuv, cfg, 1.0 * vol, torch.float32, dev, F0)
        torch.cuda.synchronize(dev)
        t1 = time.perf_counter()
        losses(xs, Fs)["spread"].backward()
        torch.cuda.synchronize(dev)
        t2 = time.perf_counter()
        r = dict(forward_s=t1 - t0, backward_s=t2 - t1, backward_ms_per_substep=(t2 - t1) / steps * 1e3,
                 dE=E.grad.item(), dnu=nuv.grad.item())
        best = r if best is None or r["backward_s"] < best["backward_s"] else best
    return dict(n=n, res=res, steps=steps, checkpoint_every=every, **best)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--n", type=int, default=131072)
    ap.add_argument("--res", type=int, default=64)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--every", type=int, default=50)
    ap.add_argument("--dt", type=float, default=1e-4)
    ap.add_argument("--E", type=float, default=4e3)
    ap.add_argument("--nu", type=float, default=0.3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--model", default="fixed_corotated", choices=("fixed_corotated", "neo_hookean"))
    ap.add_argument("--f0-std", type=float, default=0.0, help="initial deformation: F0 = I + N(0, s^2)")
    ap.add_argument("--time-backward", action="store_true",
                    help="only time the float32 forward and backward of the spread loss (no finite differences)")
    a = ap.parse_args(argv)
    if a.time_backward:
        print(json.dumps(time_backward(a.n, a.res, a.steps, a.every, a.dt, a.E, a.nu, a.seed, a.model)))
        return
    r = run(a.n, a.res, a.steps, a.every, a.dt, a.E, a.nu, a.seed, a.model, a.f0_std)
    print(json.dumps(r, indent=1, default=float))


if __name__ == "__main__":
    main()
