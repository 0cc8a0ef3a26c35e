"""GPU adjoint of the 3D substep (ffmpm_substep_adjoint) and the differentiable rollout.

* one adjoint substep through the C ABI against the FP64 numpy adjoint (oracle/adjoint3d.py,
  itself pinned by central differences), in float64 and float32;
* rollout gradients (v0 along a random direction, E, nu) of the float32 and float64 adjoints
  against FP64 central differences of the GPU forward, with a ragged last checkpoint segment;
* the differentiable configuration at full size: 131,072 particles in a cube of edge 0.25, 64^3
  grid, 2000 substeps of dt 1e-4, a checkpoint every 50, centre-of-mass loss to (0.7, 0.3, 0.5).
Relative-error bound for the float32 adjoint against FP64 finite differences: 1e-3.
"""
import numpy as np
import pytest
import torch

from oracle import adjoint3d as A3
from femflow_gb300 import diff as D
from femflow_gb300 import diff_check as DC

pytestmark = pytest.mark.gpu


def _state(rng, n, fstd=0.05):
    x = rng.uniform(0.3, 0.7, (n, 3))
    v = rng.normal(0, 0.3, (n, 3))
    F = np.eye(3)[None] + rng.normal(0, fstd, (n, 3, 3))
    C = rng.normal(0, 1.0, (n, 3, 3))
    return x, v, F, C


def _t(a, dtype):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-9), (torch.float32, 2e-3)])
@pytest.mark.parametrize("fstd,model", [(0.05, "neo_hookean"), (0.3, "neo_hookean"), (0.3, "fixed_corotated")])
def test_substep_adjoint_matches_oracle(dtype, tol, fstd, model):
    rng = np.random.default_rng(11)
    n, res = 1500, 16
    prm = A3.Params3D(res=res, dt=2e-4, volume=1e-5, lam_diagonal=model == "fixed_corotated")
    st = _state(rng, n, fstd)
    mass = rng.uniform(0.5e-5, 2e-5, n)
    mu0 = rng.uniform(300, 500, n)
    lam0 = rng.uniform(400, 800, n)
    wts = tuple(rng.normal(size=a.shape) for a in st)
    (xb, vb, Fb, Cb), mub_ref, lamb_ref = A3.backward(st, mass, mu0, lam0, prm, wts)
    cfg = D.RolloutConfig(res=res, dt=prm.dt, steps=1, volume=prm.volume, model=model)
    run = D._Runner(cfg, n, dtype, torch.device("cuda"), _t(mass, dtype), _t(mu0, dtype), _t(lam0, dtype))
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


def test_adjoint_raises_out_of_bounds():
    n, res = 64, 16
    rng = np.random.default_rng(0)
    st = list(_state(rng, n))
    st[0][5] = (0.999, 0.5, 0.5)  # stencil leaves the grid
    cfg = D.RolloutConfig(res=res, dt=1e-4, steps=1, volume=1e-5)
    run = D._Runner(cfg, n, torch.float32, torch.device("cuda"), 1e-5, _t(np.full(n, 400.0), torch.float32),
                    _t(np.full(n, 600.0), torch.float32))
    state = D.pack(*(_t(a, torch.float32) for a in st))
    adj = torch.zeros_like(state)
    z = torch.zeros(n, dtype=torch.float64, device="cuda")
    run.adjoint(state, adj, z, z.clone())
    with pytest.raises(RuntimeError):
        run.check()


def test_rollout_gradients_match_fp64_central_differences():
    # pre-strained (F0 = I + N(0, 0.05^2)) so that F - R is resolved by float32 (at strain 1e-4 the
    # spacing of float32 near 1.0 alone limits the float32 E-derivative to about 1e-3)
    r = DC.run(n=4096, res=32, steps=60, every=25, dt=2e-4, E_mod=2e3, nu=0.3, seed=1, f0_std=0.05)
    s = r["spread"]
    for k in ("dv", "dE", "dnu"):
        assert s[f"rel_fp64_vs_fd_{k}"] <= 1e-5, (k, s)
        assert s[f"rel_fp32_vs_fd_{k}"] <= 1e-3, (k, s)
    c = r["com"]
    assert c["rel_fp64_vs_fd_dv"] <= 1e-5 and c["rel_fp32_vs_fd_dv"] <= 1e-3, c
    st = r["strain"]
    for k in ("dv", "dE", "dnu"):
        assert st[f"rel_fp64_vs_fd_{k}"] <= 1e-5 and st[f"rel_fp32_vs_fd_{k}"] <= 1e-3, (k, st)
    assert c["rel_fp64_vs_closed_form_gv"] <= 1e-9 and c["rel_fp32_vs_closed_form_gv"] <= 1e-3, c
    assert c["rel_fp32_vs_fp64_gv"] <= 1e-3


def test_differentiable_configuration_full_size():
    """131,072 particles, 64^3, 2000 substeps, checkpoint every 50 (E = 4e3, nu = 0.3, textbook
    fixed-corotated stress).  The float32 adjoint meets 1e-3 against FP64 central differences for
    v0 on every loss, and for E and nu when it runs along the float64 trajectory; along its own
    float32 trajectory the E- and nu-derivatives of the material-sensitive losses differ by ~1.5%,
    which is the float32 forward's own E-response (same adjoint, different trajectory)."""
    r = DC.run(n=131072, res=64, steps=2000, every=50, dt=1e-4, E_mod=4e3, nu=0.3, seed=0)
    c = r["com"]
    assert c["rel_fp32_vs_fd_dv"] <= 1e-3 and c["rel_fp64_vs_fd_dv"] <= 1e-6, c
    assert c["rel_fp32_vs_closed_form_gv"] <= 1e-3 and c["rel_fp64_vs_closed_form_gv"] <= 1e-9, c
    assert c["rel_fp32_vs_fp64_gv"] <= 1e-3, c
    assert c["E_dE_over_loss_fp32"] <= 1e-6, c  # a free body's centre of mass ignores the material
    for name in ("spread", "strain"):
        s = r[name]
        assert s["rel_fp32_vs_fd_dv"] <= 1e-3, (name, s)
        assert s["rel_fp64_vs_fd_dv"] <= 1e-6, (name, s)
        assert s["rel_fp64_vs_fd_dE"] <= 1e-4 and s["rel_fp64_vs_fd_dnu"] <= 5e-4, (name, s)
        assert s["rel_fp32_adjoint_on_fp64_trajectory_vs_fd_dE"] <= 1e-3, (name, s)
        assert s["rel_fp32_adjoint_on_fp64_trajectory_vs_fd_dnu"] <= 1e-3, (name, s)
        assert s["rel_fp32_vs_fd_dE"] <= 3e-2 and s["rel_fp32_vs_fd_dnu"] <= 3e-2, (name, s)
