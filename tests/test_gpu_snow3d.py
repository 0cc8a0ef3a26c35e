"""3D snow model (three_d/p2g.py:57-61 exp hardening, three_d/g2p.py:48-58 singular-value clamp and
Jp update) on the GPU against the FP64 oracle.

The reference rebuilds F as U @ diag(s) @ Vh.T with numpy's Vh, which depends on LAPACK's
singular-vector signs; both the oracle and the kernels rebuild U diag(s) V^T, the decomposition of
F itself, so this path is pinned to the oracle rather than to reference outputs.
"""
import numpy as np
import pytest
import torch

import oracle as O
from gpu_helpers import TOL, close, n, t
from femflow_gb300.solvers.mpm import three_d
from femflow_gb300.solvers.mpm.particle import ParticleSet

pytestmark = pytest.mark.gpu


def scene(seed=5, N=1500, res=16):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.3, 0.7, size=(N, 3))
    vol = 0.4 ** 3 / N
    mass = np.full(N, vol)
    E, nu = 2e3, 0.25
    mu = np.full(N, E / (2 * (1 + nu)))
    lam = np.full(N, E * nu / ((1 + nu) * (1 - 2 * nu)))
    v = rng.normal(0, 0.2, size=(N, 3))
    F = np.zeros((N, 3, 3))
    for p in range(N):
        Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        F[p] = Q @ np.diag(rng.uniform(0.95, 1.03, size=3))  # outside the clamp band [0.975, 1.0075]
    C = rng.normal(0, 0.5, size=(N, 3, 3))
    Jp = rng.uniform(0.9, 1.1, size=(N, 1))
    return dict(x=x, v=v, F=F, C=C, Jp=Jp, mass=mass, mu=mu, lam=lam, vol=vol, res=res)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_snow_3d_substeps_match_oracle(dtype):
    s = scene()
    res, dt, g, h = s["res"], 1e-4, -9.8, 10.0
    dx, inv_dx = 1 / res, float(res)
    ox, ov, oF, oC, oJ = (s[k].copy() for k in ("x", "v", "F", "C", "Jp"))
    ps = ParticleSet(t(s["x"], dtype), t(s["mass"], dtype), t(s["mu"], dtype), t(s["lam"], dtype))
    gv_, gF, gC, gJ = (t(s[k], dtype) for k in ("v", "F", "C", "Jp"))
    R = res + 1
    for _ in range(3):
        # oracle, phase by phase
        Gv = np.zeros((R, R, R, 3)); Gm = np.zeros((R, R, R, 1))
        O.p2g_3d(inv_dx, h, dx, dt, s["vol"], Gv, Gm, ox, s["mass"], s["mu"], s["lam"], ov, oF, oC, oJ, "snow")
        O.grid_op_3d(res, dx, dt, g, Gv, Gm)
        O.g2p_3d(inv_dx, dt, Gv, ox, ov, oF, oC, oJ, "snow")
        # GPU, same phases
        gv = torch.zeros((R, R, R, 3), dtype=dtype, device="cuda")
        gm = torch.zeros((R, R, R, 1), dtype=dtype, device="cuda")
        three_d.p2g(inv_dx, h, dx, dt, s["vol"], gv, gm, ps, gv_, gF, gC, gJ, "snow")
        three_d.grid_op(res, dx, dt, g, gv, gm)
        three_d.g2p(inv_dx, dt, gv, ps, gv_, gF, gC, gJ, "snow")
    tol = TOL[dtype]
    vs = np.abs(ov).max()
    close(n(ps.pos), ox, 5 * tol["x"], scale=1.0, what="x")
    close(n(gv_), ov, 5 * tol["v"], scale=vs, what="v")
    close(n(gF), oF, 20 * tol["F"], scale=1.0, what="F")
    close(n(gJ), oJ, 20 * tol["F"], scale=1.0, what="Jp")
    # the clamp acted: every singular value of F is inside the band after a snow G2P
    sv = np.linalg.svd(n(gF), compute_uv=False)
    assert sv.min() > 0.975 - 1e-4 and sv.max() < 1.0075 + 1e-4


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_snow_3d_resident_solver_matches_oracle(dtype):
    """The snow model through the resident solver (fused G2P + next-substep P2G: the hardening of
    the P2G half uses the Jp its own G2P half just updated) against the oracle's substeps."""
    from femflow_gb300.solver import MPMSolver

    s = scene(seed=9)
    res, dt, g, h, steps = s["res"], 1e-4, -9.8, 10.0, 6
    solver = MPMSolver(torch.tensor(s["x"]), res=res, dt=dt, gravity=g, volume=s["vol"], hardening=h,
                       mass=torch.tensor(s["mass"]), mu_0=torch.tensor(s["mu"]), lambda_0=torch.tensor(s["lam"]),
                       v=torch.tensor(s["v"]), F=torch.tensor(s["F"]), C=torch.tensor(s["C"]),
                       Jp=torch.tensor(s["Jp"]), dtype=dtype, model="snow")
    solver.step(steps, check=True)
    got = solver.state()
    ox, ov, oF, oC, oJ = (s[k].copy() for k in ("x", "v", "F", "C", "Jp"))
    for _ in range(steps):
        O.substep_3d(res, float(res), h, 1 / res, dt, s["vol"], g, ox, s["mass"], s["mu"], s["lam"], ov, oF, oC,
                     oJ, "snow")
    tol = TOL[dtype]
    close(n(got["x"]), ox, 5 * tol["x"], scale=1.0, what="x")
    close(n(got["v"]), ov, 5 * tol["v"], scale=np.abs(ov).max(), what="v")
    close(n(got["F"]), oF, 20 * tol["F"], scale=1.0, what="F")
    close(n(got["Jp"]).reshape(-1, 1), oJ, 20 * tol["F"], scale=1.0, what="Jp")


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_snow_2d_resident_solver_matches_oracle(dtype):
    """2D snow through the resident solver against the oracle's 2D substeps (x, v, Jp; 2D F is
    defined up to the sign of LAPACK's SVD, see two_d/g2p.py:37-43)."""
    from femflow_gb300.solver import MPMSolver

    rng = np.random.default_rng(4)
    N, res, dt, g, h, steps = 1200, 32, 1e-4, -9.8, 10.0, 6
    x = rng.uniform(0.3, 0.7, (N, 2))
    vol = 0.16 / N
    E, nu = 2e3, 0.25
    mu, lam = E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))
    v = rng.normal(0, 0.2, (N, 2))
    F = np.array([np.diag(rng.uniform(0.95, 1.03, 2)) for _ in range(N)])
    C = rng.normal(0, 0.5, (N, 2, 2))
    Jp = rng.uniform(0.9, 1.1, (N, 1))
    solver = MPMSolver(torch.tensor(x), res=res, dt=dt, gravity=g, volume=vol, hardening=h, mass=vol, mu_0=mu,
                       lambda_0=lam, v=torch.tensor(v), F=torch.tensor(F), C=torch.tensor(C), Jp=torch.tensor(Jp),
                       dtype=dtype, model="snow")
    solver.step(steps, check=True)
    got = solver.state()
    ox, ov, oF, oC, oJ = x.copy(), v.copy(), F.copy(), C.copy(), Jp.copy()
    for _ in range(steps):
        O.substep_2d(res, float(res), h, mu, lam, vol, 1 / res, dt, vol, g, ox, ov, oF, oC, oJ, "snow")
    tol = TOL[dtype]
    close(n(got["x"]), ox, 5 * tol["x"], scale=1.0, what="x")
    close(n(got["v"]), ov, 5 * tol["v"], scale=np.abs(ov).max(), what="v")
    close(n(got["Jp"]).reshape(-1, 1), oJ, 20 * tol["F"], scale=1.0, what="Jp")
