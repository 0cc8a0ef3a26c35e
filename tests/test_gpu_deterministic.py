"""Deterministic P2G mode: bit-identical repeated runs, and the same answers as the default mode."""
import numpy as np
import pytest
import torch

from golden_cases import load, names
from gpu_helpers import TOL, close, n, t
from femflow_gb300.scenes import two_cubes
from femflow_gb300.solver import MPMSolver
from femflow_gb300.solvers.mpm import mls_mpm, three_d, two_d
from femflow_gb300.solvers.mpm.particle import ParticleSet

pytestmark = pytest.mark.gpu


def _solver(s, res, dtype, det):
    return MPMSolver(torch.tensor(s["x"]), res=res, dt=2e-4, gravity=-9.8, volume=s["vol"], mass=s["mass"],
                     mu_0=s["mu"], lambda_0=s["lam"], v=torch.tensor(s["v"]), dtype=dtype, deterministic=det)


def test_resident_deterministic_runs_are_bit_identical():
    s = two_cubes(20_000, E=4.5e3)
    a, b = _solver(s, 48, torch.float32, True), _solver(s, 48, torch.float32, True)
    a.step(15)
    b.step(15)
    sa, sb = a.state(), b.state()
    for k in ("x", "v", "F", "C"):
        assert torch.equal(sa[k], sb[k]), k
    a.check()


def test_drop_in_deterministic_runs_are_bit_identical():
    s = two_cubes(3_000, E=4.5e3)
    out = []
    for _ in range(2):
        ps = ParticleSet(t(s["x"], torch.float32), t(np.full(s["n"], s["mass"]), torch.float32),
                         t(np.full(s["n"], s["mu"]), torch.float32), t(np.full(s["n"], s["lam"]), torch.float32))
        v, F, C, Jp = mls_mpm.make_mls_mpm_coefficients(s["n"], 3)
        v.copy_(t(s["v"], torch.float32))
        for _ in range(6):
            mls_mpm.solve_mls_mpm_3d(32, 32.0, 1.0, 1 / 32, 2e-4, s["vol"], -9.8, ps, v, F, C, Jp, deterministic=True)
        out.append((ps.pos.clone(), v.clone(), F.clone(), C.clone()))
    for x0, x1 in zip(out[0], out[1]):
        assert torch.equal(x0, x1)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_deterministic_matches_default_mode(dtype):
    s = two_cubes(4_000, E=4.5e3)
    a, b = _solver(s, 32, dtype, True), _solver(s, 32, dtype, False)
    a.step(10)
    b.step(10)
    rel = 1e-12 if dtype == torch.float64 else 1e-5
    close(n(a.state()["x"]), n(b.state()["x"]), rel, scale=1.0, what="x det vs default")
    close(n(a.state()["F"]), n(b.state()["F"]), 10 * rel, scale=1.0, what="F det vs default")


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("name", names("ref3d_"))
def test_deterministic_p2g_matches_reference_3d(name, dtype):
    d = load(name)
    res, dx, inv_dx, dt, grav, vol, h, steps = d["params"]
    res = int(res)
    ps = ParticleSet(t(d["x0"], dtype), t(d["mass"], dtype), t(d["mu0"], dtype), t(d["lam0"], dtype))
    v, F, C, Jp = (t(d[k + "0"], dtype) for k in ("v", "F", "C", "Jp"))
    R = res + 1
    gv = torch.zeros((R, R, R, 3), dtype=dtype, device="cuda")
    gm = torch.zeros((R, R, R, 1), dtype=dtype, device="cuda")
    three_d.p2g(inv_dx, h, dx, dt, vol, gv, gm, ps, v, F, C, Jp, str(d["model"]), deterministic=True)
    close(n(gv), d["p2g_gv"], TOL[dtype]["grid"], what="det p2g momentum")
    close(n(gm), d["p2g_gm"], TOL[dtype]["grid"], what="det p2g mass")


@pytest.mark.parametrize("name", names("ref2d_"))
def test_deterministic_substeps_match_reference_2d(name):
    from gpu_helpers import sign_align
    d = load(name)
    res, dx, inv_dx, dt, grav, vol, mass, mu, lam, h, steps = d["params"]
    dtype = torch.float64
    x, v, F, C, Jp = (t(d[k + "0"], dtype) for k in ("x", "v", "F", "C", "Jp"))
    for _ in range(int(steps)):
        two_d.solve_mls_mpm_2d(int(res), inv_dx, h, mu, lam, mass, dx, dt, vol, grav, x, v, F, C, Jp,
                               str(d["model"]), deterministic=True)
    close(n(x), d["x"], 5e-12, scale=1.0, what="x")
    close(sign_align(n(F), d["F"]), d["F"], 5e-11, scale=1.0, what="F")
