"""GPU parity of the 3D path against the reference's golden vectors and the FP64 oracle."""
import numpy as np
import pytest
import torch

import oracle as O
from golden_cases import load, names
from gpu_helpers import TOL, close, n, t
from femflow_gb300.solvers.mpm import mls_mpm, three_d
from femflow_gb300.solvers.mpm.particle import ParticleSet

pytestmark = pytest.mark.gpu
DTYPES = [torch.float64, torch.float32]


def _case(name, dtype):
    d = load(name)
    res, dx, inv_dx, dt, grav, vol, h, steps = d["params"]
    ps = ParticleSet(t(d["x0"], dtype), t(d["mass"], dtype), t(d["mu0"], dtype), t(d["lam0"], dtype))
    state = [t(d[k + "0"], dtype) for k in ("v", "F", "C", "Jp")]
    return d, (int(res), dx, inv_dx, dt, grav, vol, h, int(steps)), ps, state


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("name", names("ref3d_"))
def test_three_d_phases_match_reference(name, dtype):
    d, (res, dx, inv_dx, dt, grav, vol, h, steps), ps, (v, F, C, Jp) = _case(name, dtype)
    tol = TOL[dtype]
    R = res + 1
    gv = torch.zeros((R, R, R, 3), dtype=dtype, device="cuda")
    gm = torch.zeros((R, R, R, 1), dtype=dtype, device="cuda")
    three_d.p2g(inv_dx, h, dx, dt, vol, gv, gm, ps, v, F, C, Jp, str(d["model"]))
    # momentum scale: the largest node momentum, or node mass x velocity scale when the momentum
    # is pure rounding (F = I, v = 0 leaves only the 1e-10 polar epsilon of the 2D reference)
    mscale = max(np.abs(d["p2g_gv"]).max(), np.abs(d["p2g_gm"]).max() * (np.abs(d["v0"]).max() + abs(grav * dt)))
    close(n(gv), d["p2g_gv"], tol["grid"], scale=mscale, what="p2g momentum")
    close(n(gm), d["p2g_gm"], tol["grid"], what="p2g mass")
    three_d.grid_op(res, dx, dt, grav, gv, gm)
    close(n(gv), d["grid_gv"], 10 * tol["grid"], what="grid velocity")
    three_d.g2p(inv_dx, dt, gv, ps, v, F, C, Jp, str(d["model"]))
    vs = np.abs(d["g2p_v"]).max() + abs(grav * dt)
    close(n(ps.pos), d["g2p_x"], tol["x"], scale=1.0, what="x")
    close(n(v), d["g2p_v"], tol["v"], scale=vs, what="v")
    close(n(C), d["g2p_C"], tol["C"], scale=vs * inv_dx, what="C")
    close(n(F), d["g2p_F"], tol["F"], scale=1.0, what="F")


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("name", names("ref3d_"))
def test_solve_mls_mpm_3d_matches_reference(name, dtype):
    d, (res, dx, inv_dx, dt, grav, vol, h, steps), ps, (v, F, C, Jp) = _case(name, dtype)
    tol = TOL[dtype]
    for _ in range(steps):
        mls_mpm.solve_mls_mpm_3d(res, inv_dx, h, dx, dt, vol, grav, ps, v, F, C, Jp)
    vs = np.abs(d["v"]).max() + abs(grav * dt)
    close(n(ps.pos), d["x"], 5 * tol["x"], scale=1.0, what="x")
    close(n(v), d["v"], 5 * tol["v"], scale=vs, what="v")
    close(n(C), d["C"], 5 * tol["C"], scale=vs * inv_dx, what="C")
    close(n(F), d["F"], 5 * tol["F"], scale=1.0, what="F")


def two_cubes(n_per, res, seed=0, edge=0.2, E=4.5e3, nu=0.3, speed=1.0):
    """The two-cube collision scene of the 1M-particle workload at a reduced particle count."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(-edge / 2, edge / 2, size=(n_per, 3)) + np.array([0.35, 0.5, 0.5])
    b = rng.uniform(-edge / 2, edge / 2, size=(n_per, 3)) + np.array([0.65, 0.5, 0.5])
    x = np.concatenate([a, b])
    N = len(x)
    v = np.zeros((N, 3))
    v[:n_per, 0], v[n_per:, 0] = speed, -speed
    vol = 2 * edge ** 3 / N
    mu, lam = E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))
    return dict(x=x, v=v, mass=np.full(N, vol), mu=np.full(N, mu), lam=np.full(N, lam), vol=vol, res=res)


@pytest.mark.parametrize("dtype", DTYPES)
def test_two_cube_scene_against_oracle(dtype):
    """A few thousand particles, 12 substeps of the collision scene: GPU vs the FP64 C oracle."""
    s = two_cubes(2500, 32)
    res, dt, g = s["res"], 5e-5 * 4, -9.8
    N = len(s["x"])
    x, v = s["x"].copy(), s["v"].copy()
    F = np.tile(np.eye(3), (N, 1, 1)); C = np.zeros((N, 3, 3)); Jp = np.ones((N, 1))
    ps = ParticleSet(t(x, dtype), t(s["mass"], dtype), t(s["mu"], dtype), t(s["lam"], dtype))
    gv_, gF, gC, gJ = t(v, dtype), t(F, dtype), t(C, dtype), t(Jp, dtype)
    steps = 12
    for _ in range(steps):
        O.substep_3d(res, float(res), 1.0, 1 / res, dt, s["vol"], g, x, s["mass"], s["mu"], s["lam"], v, F, C, Jp)
        mls_mpm.solve_mls_mpm_3d(res, float(res), 1.0, 1 / res, dt, s["vol"], g, ps, gv_, gF, gC, gJ)
    tol = TOL[dtype]
    close(n(ps.pos), x, 10 * tol["x"], scale=1.0, what="x")
    close(n(gv_), v, 10 * tol["v"], scale=np.abs(v).max(), what="v")
    close(n(gF), F, 10 * tol["F"], scale=1.0, what="F")
    close(n(gC), C, 10 * tol["C"], scale=np.abs(v).max() * res, what="C")


def test_out_of_bounds_raises_like_reference():
    dtype = torch.float32
    ps = ParticleSet(t([[0.5, 0.5, 0.5], [0.999, 0.5, 0.5]], dtype), t([1.0, 1.0], dtype), t([1.0, 1.0], dtype),
                     t([1.0, 1.0], dtype))
    v, F, C, Jp = mls_mpm.make_mls_mpm_coefficients(2, 3)
    with pytest.raises(RuntimeError, match="out of grid"):
        mls_mpm.solve_mls_mpm_3d(16, 16.0, 1.0, 1 / 16, 1e-4, 1.0, -9.8, ps, v, F, C, Jp)
    # the workspace status is cleared after raising: a valid call succeeds
    ps2 = ParticleSet(t([[0.5, 0.5, 0.5]], dtype), t([1.0], dtype), t([1.0], dtype), t([1.0], dtype))
    v, F, C, Jp = mls_mpm.make_mls_mpm_coefficients(1, 3)
    mls_mpm.solve_mls_mpm_3d(16, 16.0, 1.0, 1 / 16, 1e-4, 1.0, -9.8, ps2, v, F, C, Jp)


def test_empty_particle_set():
    dtype = torch.float32
    ps = ParticleSet(torch.zeros((0, 3), dtype=dtype, device="cuda"), *(torch.zeros(0, dtype=dtype, device="cuda"),) * 3)
    v, F, C, Jp = mls_mpm.make_mls_mpm_coefficients(0, 3)
    mls_mpm.solve_mls_mpm_3d(16, 16.0, 1.0, 1 / 16, 1e-4, 1.0, -9.8, ps, v, F, C, Jp)


def test_mixed_dtypes_rejected():
    ps = ParticleSet(t([[0.5, 0.5, 0.5]], torch.float32), t([1.0], torch.float32), t([1.0], torch.float32),
                     t([1.0], torch.float32))
    v, F, C, Jp = mls_mpm.make_mls_mpm_coefficients(1, 3, dtype=torch.float64)
    with pytest.raises(TypeError):
        mls_mpm.solve_mls_mpm_3d(16, 16.0, 1.0, 1 / 16, 1e-4, 1.0, -9.8, ps, v, F, C, Jp)


def test_host_arrays_are_staged_and_written_back():
    """numpy float64 arrays in, as the numba reference takes them: results land in place."""
    d = load("ref3d_drop_small")
    res, dx, inv_dx, dt, grav, vol, h, steps = d["params"]
    from femflow_gb300.solvers.mpm.particle import Particle
    plist = [Particle(d["x0"][i].copy(), 0.0, d["mass"][i], d["lam0"][i], d["mu0"][i]) for i in range(len(d["x0"]))]
    v, F, C, Jp = (d[k + "0"].copy() for k in ("v", "F", "C", "Jp"))
    for _ in range(int(steps)):
        mls_mpm.solve_mls_mpm_3d(int(res), inv_dx, h, dx, dt, vol, grav, plist, v, F, C, Jp)
    close(np.array([p.pos for p in plist]), d["x"], 1e-12, scale=1.0, what="x (host)")
    close(v, d["v"], 1e-10, scale=np.abs(d["v"]).max() + 1e-3, what="v (host)")


@pytest.mark.parametrize("dtype", DTYPES)
def test_fixed_corotated_model_against_oracle(dtype):
    """The textbook fixed-corotated stress (lam(J-1)J on the diagonal; not a reference model):
    P2G, grid update and G2P through the reference-shaped API against the FP64 C oracle."""
    rng = np.random.default_rng(7)
    N, res, dt, g, vol = 3000, 32, 2e-4, -9.8, 1e-5
    x = rng.uniform(0.3, 0.7, (N, 3)); v = rng.normal(0, 0.3, (N, 3))
    F = np.eye(3)[None] + rng.normal(0, 0.05, (N, 3, 3)); C = rng.normal(0, 1.0, (N, 3, 3)); Jp = np.ones((N, 1))
    mass, mu, lam = np.full(N, 1e-5), np.full(N, 400.0), np.full(N, 600.0)
    gv = np.zeros((res + 1,) * 3 + (3,)); gm = np.zeros((res + 1,) * 3 + (1,))
    ps = ParticleSet(t(x, dtype), t(mass, dtype), t(mu, dtype), t(lam, dtype))
    dv, dF, dC, dJ = t(v, dtype), t(F, dtype), t(C, dtype), t(Jp, dtype)
    dgv, dgm = t(gv, dtype), t(gm, dtype)
    O.p2g_3d(float(res), 1.0, 1 / res, dt, vol, gv, gm, x, mass, mu, lam, v, F, C, Jp, model="fixed_corotated")
    three_d.p2g(float(res), 1.0, 1 / res, dt, vol, dgv, dgm, ps, dv, dF, dC, dJ, "fixed_corotated")
    tol = TOL[dtype]
    close(n(dgv), gv, tol["grid"], scale=np.abs(gv).max(), what="momentum")
    close(n(dgm), gm, tol["grid"], what="mass")
    O.grid_op_3d(res, 1 / res, dt, g, gv, gm)
    three_d.grid_op(res, 1 / res, dt, g, dgv, dgm)
    O.g2p_3d(float(res), dt, gv, x, v, F, C, Jp, model="fixed_corotated")
    three_d.g2p(float(res), dt, dgv, ps, dv, dF, dC, dJ, "fixed_corotated")
    close(n(ps.pos), x, tol["x"], scale=1.0, what="x")
    close(n(dv), v, tol["v"], scale=np.abs(v).max(), what="v")
    close(n(dF), F, tol["F"], scale=1.0, what="F")
    close(n(dC), C, tol["C"], scale=np.abs(C).max(), what="C")
