"""GPU parity of the 2D path (two_d.*) against the reference's golden vectors, KATs and oracle."""
import numpy as np
import pytest
import torch

import oracle as O
from golden_cases import load, names
from gpu_helpers import TOL, close, n, sign_align, t
from femflow_gb300.solvers.mpm import two_d

pytestmark = pytest.mark.gpu
DTYPES = [torch.float64, torch.float32]


def _case(name, dtype):
    d = load(name)
    res, dx, inv_dx, dt, grav, vol, mass, mu, lam, h, steps = d["params"]
    state = [t(d[k + "0"], dtype) for k in ("x", "v", "F", "C", "Jp")]
    return d, (int(res), dx, inv_dx, dt, grav, vol, mass, mu, lam, h, int(steps)), state


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("name", names("ref2d_"))
def test_two_d_phases_match_reference(name, dtype):
    d, (res, dx, inv_dx, dt, grav, vol, mass, mu, lam, h, steps), (x, v, F, C, Jp) = _case(name, dtype)
    tol, model = TOL[dtype], str(d["model"])
    R = res + 1
    gv = torch.zeros((R, R, 2), dtype=dtype, device="cuda")
    gm = torch.zeros((R, R, 1), dtype=dtype, device="cuda")
    two_d.p2g(inv_dx, h, mu, lam, mass, dx, dt, vol, gv, gm, x, v, F, C, Jp, model)
    # momentum scale: the largest node momentum, or node mass x velocity scale when the momentum
    # is pure rounding (F = I, v = 0 leaves only the 1e-10 polar epsilon of the 2D reference)
    mscale = max(np.abs(d["p2g_gv"]).max(), np.abs(d["p2g_gm"]).max() * (np.abs(d["v0"]).max() + abs(grav * dt)))
    close(n(gv), d["p2g_gv"], tol["grid"], scale=mscale, what="p2g momentum")
    close(n(gm), d["p2g_gm"], tol["grid"], what="p2g mass")
    two_d.grid_op(res, dt, grav, gv, gm)
    close(n(gv), d["grid_gv"], 10 * tol["grid"], what="grid velocity")
    two_d.g2p(inv_dx, dt, gv, x, v, F, C, Jp, model)
    vs = np.abs(d["g2p_v"]).max() + abs(grav * dt)
    close(n(x), d["g2p_x"], tol["x"], scale=1.0, what="x")
    close(n(v), d["g2p_v"], tol["v"], scale=vs, what="v")
    close(n(C), d["g2p_C"], tol["C"], scale=vs * inv_dx, what="C")
    close(sign_align(n(F), d["g2p_F"]), d["g2p_F"], tol["F"], scale=1.0, what="F (up to sign)")
    close(n(Jp), d["g2p_Jp"], tol["Jp"], scale=1.0, what="Jp")


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("name", names("ref2d_"))
def test_two_d_substeps_match_reference(name, dtype):
    d, (res, dx, inv_dx, dt, grav, vol, mass, mu, lam, h, steps), (x, v, F, C, Jp) = _case(name, dtype)
    tol, model = TOL[dtype], str(d["model"])
    for _ in range(steps):
        two_d.solve_mls_mpm_2d(res, inv_dx, h, mu, lam, mass, dx, dt, vol, grav, x, v, F, C, Jp, model)
    vs = np.abs(d["v"]).max() + abs(grav * dt)
    close(n(x), d["x"], 5 * tol["x"], scale=1.0, what="x")
    close(n(v), d["v"], 5 * tol["v"], scale=vs, what="v")
    close(n(C), d["C"], 5 * tol["C"], scale=vs * inv_dx, what="C")
    close(sign_align(n(F), d["F"]), d["F"], 5 * tol["F"], scale=1.0, what="F (up to sign)")
    close(n(Jp), d["Jp"], 5 * tol["Jp"], scale=1.0, what="Jp")


def test_kat_p2g_grid_and_full_step_2d():
    """The reference's own (stale) MPM known-answer tests, on the GPU in float64."""
    d = load("kat")
    E, nu, mu, lam, res, dx, dt, grav, mass, vol, h = d["kat_params"]
    res, dtype = int(res), torch.float64
    x = t(d["p2g_x"], dtype)
    nn = x.shape[0]
    v = torch.zeros((nn, 2), dtype=dtype, device="cuda")
    F = torch.eye(2, dtype=dtype, device="cuda").repeat(nn, 1, 1).contiguous()
    C = torch.zeros((nn, 2, 2), dtype=dtype, device="cuda")
    Jp = torch.ones((nn, 1), dtype=dtype, device="cuda")
    gv = torch.zeros((res + 1, res + 1, 2), dtype=dtype, device="cuda")
    gm = torch.zeros((res + 1, res + 1, 1), dtype=dtype, device="cuda")
    two_d.p2g(1 / dx, h, mu, lam, mass, dx, dt, vol, gv, gm, x, v, F, C, Jp)
    close(n(gv), d["p2g_gv_ref"], 1e-12, what="KAT grid momentum")
    close(n(gm), d["p2g_gm_ref"], 1e-15, what="KAT grid mass")
    nz = n(gm)[..., 0] > 0
    got = np.concatenate([n(gv)[nz], n(gm)[nz]], axis=1)
    key = lambda a: a[np.lexsort(a.T[::-1])]
    np.testing.assert_allclose(key(np.round(got, 6)), key(d["p2g_ground_truth"]), atol=1e-6)  # ground_truth_grid.txt
    two_d.grid_op(res, dt, grav, gv, gm)
    two_d.g2p(1 / dx, dt, gv, x, v, F, C, Jp)
    close(n(x), d["step_x_ref"], 1e-14, scale=1.0, what="KAT x")
    assert np.isclose(n(x), d["step_x_expected"]).all()  # test_grid_to_particle.py expectations
    assert np.isclose(n(v), d["step_v_expected"]).all()


@pytest.mark.parametrize("dtype", DTYPES)
def test_c1_scene_against_oracle(dtype):
    """The 2D block-drop scene (8,192 particles, 128^2 grid) for 25 substeps at dt=5e-5 vs the oracle."""
    rng = np.random.default_rng(0)
    N, res, dt, g = 8192, 128, 5e-5, -9.8
    x = rng.uniform((0.3, 0.4), (0.6, 0.7), size=(N, 2))
    vol = 0.09 / N
    mass = vol
    E_, nu = 1e4, 0.2
    mu, lam = E_ / (2 * (1 + nu)), E_ * nu / ((1 + nu) * (1 - 2 * nu))
    v = np.zeros((N, 2)); F = np.tile(np.eye(2), (N, 1, 1)); C = np.zeros((N, 2, 2)); Jp = np.ones((N, 1))
    gx, gvv, gF, gC, gJ = (t(a, dtype) for a in (x, v, F, C, Jp))
    for _ in range(25):
        O.substep_2d(res, float(res), 1.0, mu, lam, mass, 1 / res, dt, vol, g, x, v, F, C, Jp)
        two_d.solve_mls_mpm_2d(res, float(res), 1.0, mu, lam, mass, 1 / res, dt, vol, g, gx, gvv, gF, gC, gJ)
    tol = TOL[dtype]
    close(n(gx), x, 10 * tol["x"], scale=1.0, what="x")
    close(n(gvv), v, 10 * tol["v"], scale=np.abs(v).max(), what="v")
    close(sign_align(n(gF), F), F, 10 * tol["F"], scale=1.0, what="F")


@pytest.mark.parametrize("dtype", DTYPES)
def test_fixed_corotated_model_against_oracle(dtype):
    """The textbook fixed-corotated stress (not a reference model), 2D phases vs the FP64 C oracle."""
    rng = np.random.default_rng(8)
    N, res, dt, g, vol, mass, mu, lam = 4000, 64, 1e-4, -9.8, 1e-5, 1e-5, 400.0, 600.0
    x = rng.uniform(0.2, 0.8, (N, 2)); v = rng.normal(0, 0.3, (N, 2))
    F = np.eye(2)[None] + rng.normal(0, 0.05, (N, 2, 2)); C = rng.normal(0, 1.0, (N, 2, 2)); Jp = np.ones((N, 1))
    gv = np.zeros((res + 1, res + 1, 2)); gm = np.zeros((res + 1, res + 1, 1))
    dx_, dv, dF, dC, dJ, dgv, dgm = (t(a, dtype) for a in (x, v, F, C, Jp, gv, gm))
    O.p2g_2d(float(res), 1.0, mu, lam, mass, 1 / res, dt, vol, gv, gm, x, v, F, C, Jp, model="fixed_corotated")
    two_d.p2g(float(res), 1.0, mu, lam, mass, 1 / res, dt, vol, dgv, dgm, dx_, dv, dF, dC, dJ, "fixed_corotated")
    tol = TOL[dtype]
    close(n(dgv), gv, tol["grid"], scale=np.abs(gv).max(), what="momentum")
    O.grid_op_2d(res, dt, g, gv, gm)
    two_d.grid_op(res, dt, g, dgv, dgm)
    O.g2p_2d(float(res), dt, gv, x, v, F, C, Jp, model="fixed_corotated")
    two_d.g2p(float(res), dt, dgv, dx_, dv, dF, dC, dJ, "fixed_corotated")
    close(n(dx_), x, tol["x"], scale=1.0, what="x")
    close(n(dv), v, tol["v"], scale=np.abs(v).max(), what="v")
    close(sign_align(n(dF), F), F, tol["F"], scale=1.0, what="F")
