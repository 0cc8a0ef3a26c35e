"""Planar colliders (three_d/grid_op.py:50-67 check_collision_points) on the GPU.

* the drop-in ``three_d.check_collision_points`` (reference's literal rule by default) against the
  reference's own output on the committed fixtures (tests/golden/colliders.npz), float64/float32;
* the "sticky" rule, more planes than one launch takes, and the 2D form against the oracle;
* planes inside the resident solver's grid update against the per-phase composition p2g ->
  grid_op -> check_collision_points -> g2p;
* the adjoint through a collider against float64 central differences of the GPU forward.
"""
import ctypes
import os

import numpy as np
import pytest
import torch

from femflow_gb300 import _native as N
from femflow_gb300 import diff as D
from femflow_gb300 import engine as E
from femflow_gb300.solver import MPMSolver
from femflow_gb300.solvers.mpm import three_d
from femflow_gb300.solvers.mpm.particle import ParticleSet
from oracle import colliders as OC

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "colliders.npz")


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_drop_in_matches_reference_fixture(dtype):
    d = np.load(GOLDEN)
    for c in "ab":
        gv = torch.tensor(d[f"{c}_grid_in"], dtype=dtype, device="cuda")
        three_d.check_collision_points(d[f"{c}_points"], d[f"{c}_normals"], int(d[f"{c}_res"]),
                                       float(d[f"{c}_dx"]), gv)
        want = torch.tensor(d[f"{c}_grid_out"], dtype=dtype)
        assert torch.equal(gv.cpu(), want)


def test_sticky_rule_and_many_planes_against_oracle():
    rng = np.random.default_rng(5)
    res, dx = 20, 1 / 20
    points = rng.uniform(0.1, 0.9, (12, 3))  # more planes than one launch carries (8)
    normals = rng.normal(size=(12, 3))
    mask, dots = OC.behind(points, normals, res, dx, 3, "sticky")
    assert np.abs(dots).min() > 1e-9  # no node on a plane: the float64 sign test is unambiguous
    gv0 = rng.normal(size=(res + 1, res + 1, res + 1, 3))
    gv = torch.tensor(gv0, device="cuda")
    three_d.check_collision_points(points, normals, res, dx, gv, rule="sticky")
    want = gv0.reshape(-1, 3).copy()
    want[mask] = 0.0
    assert np.array_equal(gv.cpu().numpy().reshape(-1, 3), want)


def test_2d_form_against_oracle():
    rng = np.random.default_rng(6)
    res, dx = 32, 1 / 32
    points, normals = rng.uniform(0.2, 0.8, (3, 2)), rng.normal(size=(3, 2))
    for rule in ("reference_literal", "sticky"):
        mask, dots = OC.behind(points, normals, res, dx, 2, rule)
        assert np.abs(dots).min() > 1e-9
        gv0 = rng.normal(size=(res + 1, res + 1, 2))
        gv = torch.tensor(gv0, dtype=torch.float32, device="cuda")
        prm = E.make_params(2, res, torch.float32, dx, 1 / dx, 1.0, plane_rule=rule)
        pts, nrm = np.ascontiguousarray(points), np.ascontiguousarray(normals)
        N.call("ffmpm_check_collision_points", ctypes.byref(prm), pts.ctypes.data_as(ctypes.c_void_p),
               nrm.ctypes.data_as(ctypes.c_void_p), 3, ctypes.c_void_p(gv.data_ptr()),
               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        want = gv0.astype(np.float32).reshape(-1, 2).copy()
        want[mask] = 0.0
        assert np.array_equal(gv.cpu().numpy().reshape(-1, 2), want)


def _block_over_plane(n=3000, res=48):
    rng = np.random.default_rng(7)
    x = rng.uniform(-0.06, 0.06, (n, 3)) + [0.5, 0.40, 0.5]  # lowest stencils reach behind the plane
    v = np.tile([[0.3, -3.0, 0.2]], (n, 1))
    vol = 0.12 ** 3 / n
    E_, nu = 3e3, 0.3
    mu, lam = E_ / (2 * (1 + nu)), E_ * nu / ((1 + nu) * (1 - 2 * nu))
    planes = [((0.5, 0.33, 0.5), (0.15, 1.0, -0.1))]  # a slightly tilted floor under the block
    return x, v, vol, mu, lam, planes, res


def test_solver_planes_match_per_phase_composition():
    x, v, vol, mu, lam, planes, res = _block_over_plane()
    n, dt, g, steps = len(x), 2e-4, -9.8, 40
    solver = MPMSolver(torch.tensor(x), res=res, dt=dt, gravity=g, volume=vol, mass=vol, mu_0=mu, lambda_0=lam,
                       v=torch.tensor(v), dtype=torch.float64, planes=planes)
    solver.step(steps, check=True)
    got = solver.state()
    free = MPMSolver(torch.tensor(x), res=res, dt=dt, gravity=g, volume=vol, mass=vol, mu_0=mu, lambda_0=lam,
                     v=torch.tensor(v), dtype=torch.float64)
    free.step(steps, check=True)
    t = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    ps = ParticleSet(t(x), t(np.full(n, vol)), t(np.full(n, mu)), t(np.full(n, lam)))
    vv = t(v)
    F = t(np.tile(np.eye(3), (n, 1, 1)))
    C = torch.zeros((n, 3, 3), dtype=torch.float64, device="cuda")
    Jp = torch.ones((n, 1), dtype=torch.float64, device="cuda")
    R = res + 1
    pts = np.array([p for p, _ in planes])
    nrm = np.array([q for _, q in planes])
    for _ in range(steps):
        gv = torch.zeros((R, R, R, 3), dtype=torch.float64, device="cuda")
        gm = torch.zeros((R, R, R, 1), dtype=torch.float64, device="cuda")
        three_d.p2g(float(res), 1.0, 1 / res, dt, vol, gv, gm, ps, vv, F, C, Jp)
        three_d.grid_op(res, 1 / res, dt, g, gv, gm)
        three_d.check_collision_points(pts, nrm, res, 1 / res, gv, rule="sticky")
        three_d.g2p(float(res), dt, gv, ps, vv, F, C, Jp)
    xs, xw = got["x"].cpu().numpy(), ps.pos.cpu().numpy()
    np.testing.assert_allclose(xs, xw, rtol=0, atol=1e-12)
    np.testing.assert_allclose(got["v"].cpu().numpy(), vv.cpu().numpy(), rtol=0, atol=1e-9)
    # the collider stopped the block's lower layer: the free block fell further
    assert (free.state()["x"][:, 1].min() - got["x"][:, 1].min()).item() < -1e-3


def test_adjoint_through_a_collider_matches_central_differences():
    x, v, vol, mu, lam, planes, res = _block_over_plane(n=1500, res=32)
    cfg = D.RolloutConfig(res=res, dt=2e-4, steps=12, volume=vol, checkpoint_every=5, planes=tuple(planes))
    t = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    x0, v0 = t(x), t(v)
    rng = np.random.default_rng(8)
    direction = t(rng.normal(size=v.shape))
    w = t(rng.normal(size=(3,)))

    def loss(v_init):
        xe, ve, _, _ = D.simulate(x0, v_init, mu, lam, cfg, vol)
        return (xe.mean(0) * w).sum() + 0.1 * (ve ** 2).mean()

    vg = v0.clone().requires_grad_(True)
    loss(vg).backward()
    ad = float((vg.grad * direction).sum())
    eps = 1e-5
    fd = (float(loss(v0 + eps * direction)) - float(loss(v0 - eps * direction))) / (2 * eps)
    assert abs(ad - fd) <= 1e-6 * max(abs(fd), 1e-12), (ad, fd)


def test_2d_solver_planes_match_per_phase_composition():
    """2D resident solver with a plane against two_d.p2g -> grid_op -> the collider -> g2p (float64;
    x and v: 2D F is defined up to the sign of LAPACK's SVD, two_d/g2p.py:37-43)."""
    from femflow_gb300.solvers.mpm import two_d

    rng = np.random.default_rng(12)
    n, res, dt, g, steps = 2000, 48, 2e-4, -9.8, 30
    x = rng.uniform(-0.06, 0.06, (n, 2)) + [0.5, 0.40]
    v = np.tile([[0.3, -3.0]], (n, 1))
    vol = 0.12 ** 2 / n
    E_, nu = 3e3, 0.3
    mu, lam = E_ / (2 * (1 + nu)), E_ * nu / ((1 + nu) * (1 - 2 * nu))
    planes = [((0.5, 0.33), (0.15, 1.0))]
    solver = MPMSolver(torch.tensor(x), res=res, dt=dt, gravity=g, volume=vol, mass=vol, mu_0=mu, lambda_0=lam,
                       v=torch.tensor(v), dtype=torch.float64, planes=planes)
    solver.step(steps, check=True)
    got = solver.state()
    t = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    gx, gvv = t(x), t(v)
    gF, gC, gJ = t(np.tile(np.eye(2), (n, 1, 1))), t(np.zeros((n, 2, 2))), t(np.ones((n, 1)))
    R = res + 1
    prm = E.make_params(2, res, torch.float64, 1 / res, float(res), dt, plane_rule="sticky")
    pts = np.ascontiguousarray([p for p, _ in planes], dtype=np.float64)
    nrm = np.ascontiguousarray([q for _, q in planes], dtype=np.float64)
    for _ in range(steps):
        gv = torch.zeros((R, R, 2), dtype=torch.float64, device="cuda")
        gm = torch.zeros((R, R, 1), dtype=torch.float64, device="cuda")
        two_d.p2g(float(res), 1.0, mu, lam, vol, 1 / res, dt, vol, gv, gm, gx, gvv, gF, gC, gJ)
        two_d.grid_op(res, dt, g, gv, gm)
        N.call("ffmpm_check_collision_points", ctypes.byref(prm), pts.ctypes.data_as(ctypes.c_void_p),
               nrm.ctypes.data_as(ctypes.c_void_p), 1, ctypes.c_void_p(gv.data_ptr()),
               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        two_d.g2p(float(res), dt, gv, gx, gvv, gF, gC, gJ)
    np.testing.assert_allclose(got["x"].cpu().numpy(), gx.cpu().numpy(), rtol=0, atol=1e-12)
    np.testing.assert_allclose(got["v"].cpu().numpy(), gvv.cpu().numpy(), rtol=0, atol=1e-9)
