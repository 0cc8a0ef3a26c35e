"""GPU adjoint of the 2D substep (ffmpm_substep_adjoint with dim 2) and the 2D differentiable rollout.

* one adjoint substep through the C ABI against the FP64 numpy adjoint (oracle/adjoint2d.py,
  itself pinned by central differences), in float64 and float32, away from and along the 0.05
  wall band;
* rollout gradients (v0 along a random direction, E, nu) of the float64 and float32 adjoints
  against FP64 central differences of the GPU forward, with a ragged last checkpoint segment.
Relative-error bound for the float32 rollout gradients against FP64 finite differences: 1e-3.
"""
import numpy as np
import pytest
import torch

from oracle import adjoint2d as A2
from femflow_gb300 import diff as D

pytestmark = pytest.mark.gpu


def _state(rng, n, fstd=0.05, lo=0.2, hi=0.8):
    x = rng.uniform(lo, hi, (n, 2))
    v = rng.normal(0, 0.3, (n, 2))
    F = np.eye(2)[None] + rng.normal(0, fstd, (n, 2, 2))
    C = rng.normal(0, 1.0, (n, 2, 2))
    return x, v, F, C


def _t(a, dtype):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-9), (torch.float32, 2e-3)])
@pytest.mark.parametrize("fstd,model,lo,hi", [(0.05, "neo_hookean", 0.2, 0.8), (0.3, "neo_hookean", 0.2, 0.8),
                                              (0.3, "fixed_corotated", 0.2, 0.8),
                                              (0.05, "neo_hookean", 0.02, 0.98)])
def test_substep_adjoint2d_matches_oracle(dtype, tol, fstd, model, lo, hi):
    rng = np.random.default_rng(21)
    n, res = 2000, 32
    prm = A2.Params2D(res=res, dt=2e-4, volume=1e-4, lam_diagonal=model == "fixed_corotated")
    st = _state(rng, n, fstd, lo, hi)
    mass = rng.uniform(0.5e-4, 2e-4, n)
    mu0 = rng.uniform(300, 500, n)
    lam0 = rng.uniform(400, 800, n)
    wts = tuple(rng.normal(size=a.shape) for a in st)
    (xb, vb, Fb, Cb), mub_ref, lamb_ref = A2.backward(st, mass, mu0, lam0, prm, wts)
    cfg = D.RolloutConfig(res=res, dt=prm.dt, steps=1, volume=prm.volume, model=model)
    run = D._Runner(cfg, n, dtype, torch.device("cuda"), _t(mass, dtype), _t(mu0, dtype), _t(lam0, dtype), dim=2)
    state = D.pack(*(_t(a, dtype) for a in st))
    adj = D.pack(*(_t(a, dtype) for a in wts))
    mub = torch.zeros(n, dtype=torch.float64, device="cuda")
    lamb = torch.zeros(n, dtype=torch.float64, device="cuda")
    run.adjoint(state, adj, mub, lamb)
    run.check()
    got = D.unpack(adj)
    for g, want, name in zip(got, (xb, vb, Fb, Cb), "xvFC"):
        g = g.double().cpu().numpy()
        err = np.abs(g - want).max() / np.abs(want).max()
        assert err <= tol, (name, err)
    for g, want, name in ((mub, mub_ref, "mu"), (lamb, lamb_ref, "lam")):
        err = np.abs(g.cpu().numpy() - want).max() / np.abs(want).max()
        assert err <= tol, (name, err)


def _spread(x):
    x = x.double()
    return ((x - x.mean(dim=0)) ** 2).sum(dim=1).mean()


def _scene(n, seed):
    rng = np.random.default_rng(seed)
    x0 = rng.uniform(0.35, 0.65, (n, 2))
    v0 = rng.normal(0.0, 0.2, (n, 2))
    F0 = np.eye(2)[None] + rng.normal(0.0, 0.05, (n, 2, 2))  # pre-strained, as the 3D check
    direction = rng.normal(0.0, 1.0, (n, 2))
    return x0, v0, F0, direction


def _loss(x0, v0, F0, E, nu, cfg, mass, dtype, grad=False):
    mu, lam = D.lame(E, nu)
    x = _t(x0, dtype)
    v = v0 if torch.is_tensor(v0) else _t(v0, dtype)
    xs, _, _, _ = D.simulate(x, v, mu.to(dtype), lam.to(dtype), cfg, mass, F0=_t(F0, dtype))
    return _spread(xs)


def test_rollout2d_gradients_match_fp64_central_differences():
    n = 4096
    x0, v0, F0, direction = _scene(n, 3)
    vol = 0.3 * 0.3 / n
    cfg = D.RolloutConfig(res=64, dt=2e-4, steps=60, volume=vol, checkpoint_every=25)
    mass = 1.0 * vol
    E0, nu0 = 2e3, 0.3
    grads = {}
    for dtype in (torch.float64, torch.float32):
        E = torch.tensor(E0, dtype=torch.float64, device="cuda", requires_grad=True)
        nu = torch.tensor(nu0, dtype=torch.float64, device="cuda", requires_grad=True)
        v = _t(v0, dtype).requires_grad_(True)
        L = _loss(x0, v, F0, E, nu, cfg, mass, dtype)
        L.backward()
        gv = float((v.grad.double().cpu().numpy() * direction).sum())
        grads[dtype] = dict(dv=gv, dE=E.grad.item(), dnu=nu.grad.item())
    with torch.no_grad():
        f = lambda v, E, nu: _loss(x0, v, F0, torch.tensor(E, dtype=torch.float64, device="cuda"),
                                   torch.tensor(nu, dtype=torch.float64, device="cuda"), cfg, mass,
                                   torch.float64).item()
        hv, hE, hnu = 1e-4, 1e-4 * E0, 1e-4
        fd = dict(dv=(f(v0 + hv * direction, E0, nu0) - f(v0 - hv * direction, E0, nu0)) / (2 * hv),
                  dE=(f(v0, E0 + hE, nu0) - f(v0, E0 - hE, nu0)) / (2 * hE),
                  dnu=(f(v0, E0, nu0 + hnu) - f(v0, E0, nu0 - hnu)) / (2 * hnu))
    for k in ("dv", "dE", "dnu"):
        r64 = abs(grads[torch.float64][k] - fd[k]) / abs(fd[k])
        r32 = abs(grads[torch.float32][k] - fd[k]) / abs(fd[k])
        assert r64 <= 1e-5, (k, r64, grads, fd)
        assert r32 <= 1e-3, (k, r32, grads, fd)


@pytest.mark.parametrize("dim", [2, 3])
def test_adjoint_of_no_particles_is_a_no_op(dim):
    cfg = D.RolloutConfig(res=16, dt=1e-4, steps=1, volume=1e-5)
    z = torch.zeros(0, dtype=torch.float32, device="cuda")
    run = D._Runner(cfg, 0, torch.float32, torch.device("cuda"), 1e-5, z, z, dim=dim)
    rows = 24 if dim == 3 else 12
    state = torch.zeros((rows, 0), dtype=torch.float32, device="cuda")
    adj = torch.zeros_like(state)
    run.adjoint(state, adj, torch.zeros(0, dtype=torch.float64, device="cuda"),
                torch.zeros(0, dtype=torch.float64, device="cuda"))
    run.check()


def test_rollout2d_of_one_particle_has_gradients():
    cfg = D.RolloutConfig(res=32, dt=1e-4, steps=5, volume=1e-4, checkpoint_every=2)
    x = torch.tensor([[0.5, 0.6]], dtype=torch.float64, device="cuda")
    v = torch.tensor([[0.1, -0.2]], dtype=torch.float64, device="cuda", requires_grad=True)
    xs, vs, _, _ = D.simulate(x, v, torch.tensor(400.0, dtype=torch.float64), torch.tensor(600.0, dtype=torch.float64),
                              cfg, 1e-4)
    xs[:, 0].sum().backward()
    # a lone particle moves ballistically under gravity: dx/dv0 = total time along x
    assert abs(float(v.grad[0, 0]) - 5 * 1e-4) < 1e-9
