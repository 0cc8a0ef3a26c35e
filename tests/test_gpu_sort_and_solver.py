"""Block sort bit-exactness, the resident sorted solver, CUDA-graph replay and FP64 diagnostics."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_helpers import close, n, t
from femflow_gb300 import _native as N
from femflow_gb300 import engine as E
from femflow_gb300.solver import MPMSolver
from femflow_gb300.solvers.mpm import mls_mpm
from femflow_gb300.solvers.mpm.particle import ParticleSet
from test_gpu_parity_3d import two_cubes

pytestmark = pytest.mark.gpu


def host_keys(x32, res, bs, det):
    """Block keys computed on the host with the kernels' rounding (float32 mul, then sub)."""
    xs = (x32 * np.float32(res)).astype(np.float32)
    tt = (xs - np.float32(0.5)).astype(np.float32)
    valid = np.all((tt > -1) & (tt < res), axis=1)
    b = np.where(valid[:, None], np.trunc(tt), 0).astype(np.int64)
    valid &= np.all((b >= 0) & (b + 2 <= res), axis=1)
    R = res + 1
    nb = (R + bs - 1) // bs
    blk = np.zeros(len(x32), dtype=np.int64)
    cell = np.zeros(len(x32), dtype=np.int64)
    for dd in range(x32.shape[1]):
        blk = blk * nb + b[:, dd] // bs
        cell = cell * bs + b[:, dd] % bs
    cbits = x32.shape[1] * int(np.log2(bs))  # keys order by block, then by cell inside the block
    key = (blk << cbits) | cell
    key = np.where(valid, key, 0xFFFFFFFF).astype(np.uint64)
    return key


@pytest.mark.parametrize("dim,res,det", [(3, 64, False), (3, 128, False), (3, 64, True), (2, 128, False), (2, 256, True)])
def test_sort_by_block_is_bit_exact_stable(dim, res, det):
    rng = np.random.default_rng(7)
    nn = 200_003
    x = rng.uniform(0.05, 0.95, size=(nn, dim)).astype(np.float32)
    x[::997] = 1.5  # out of the grid: key 0xFFFFFFFF, sorted last
    prm = E.make_params(dim, res, torch.float32, 1 / res, float(res), 1e-4, deterministic=det)
    ws = E.Workspace(prm, nn, "cuda")
    xd = torch.from_numpy(x).cuda()
    keys = torch.empty(nn, dtype=torch.int32, device="cuda")
    perm = torch.empty(nn, dtype=torch.int32, device="cuda")
    N.call("ffmpm_sort_by_block", ctypes.byref(prm), ctypes.c_void_p(xd.data_ptr()), nn,
           ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(ws.ptr),
           ctypes.c_size_t(ws.bytes), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    bs = (8 if not det else 4) if dim == 3 else (16 if not det else 8)
    hk = host_keys(x, res, bs, det)
    ref_perm = np.argsort(hk, kind="stable")
    got_keys = keys.cpu().numpy().view(np.uint32).astype(np.uint64)
    assert np.array_equal(got_keys, hk[ref_perm])
    assert np.array_equal(perm.cpu().numpy().astype(np.int64), ref_perm)
    st, _ = ws.status()
    assert st & N.STATUS_OOB  # the planted out-of-grid particles are reported


def _scene(dtype, n_per=3000, res=32):
    s = two_cubes(n_per, res)
    return s


# variant 0 runs the fused G2P + P2G kernel, 4 separate G2P and P2G launches, 1 and 2 the P2G variants
@pytest.mark.parametrize("variant,sort_every", [(0, 1), (1, 1), (2, 1), (0, 3), (0, 8), (4, 1), (4, 8)])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_sorted_solver_matches_in_place_substeps(dtype, variant, sort_every):
    s = _scene(dtype)
    res, dt, g, steps = s["res"], 2e-4, -9.8, 10
    solver = MPMSolver(torch.tensor(s["x"]), res=res, dt=dt, gravity=g, volume=s["vol"],
                       mass=torch.tensor(s["mass"]), mu_0=torch.tensor(s["mu"]), lambda_0=torch.tensor(s["lam"]),
                       v=torch.tensor(s["v"]), dtype=dtype, variant=variant, sort_every=sort_every)
    solver.step(steps, check=True)
    got = solver.state()
    N_ = len(s["x"])
    ps = ParticleSet(t(s["x"], dtype), t(s["mass"], dtype), t(s["mu"], dtype), t(s["lam"], dtype))
    v, F, C, Jp = mls_mpm.make_mls_mpm_coefficients(N_, 3, dtype=dtype)
    v.copy_(t(s["v"], dtype))
    for _ in range(steps):
        mls_mpm.solve_mls_mpm_3d(res, float(res), 1.0, 1 / res, dt, s["vol"], g, ps, v, F, C, Jp)
    rel = 1e-12 if dtype == torch.float64 else 1e-5
    close(n(got["x"]), n(ps.pos), rel, scale=1.0, what="x")
    close(n(got["v"]), n(v), 50 * rel, scale=1.0, what="v")
    close(n(got["F"]), n(F), 10 * rel, scale=1.0, what="F")
    # the ids are a permutation and the state stays sorted by block
    ids = solver.sorted_state()["ids"].cpu().numpy()
    assert np.array_equal(np.sort(ids), np.arange(N_))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_fast_particles_between_sorts(dtype):
    """A cube crossing several blocks between scheduled re-sorts (25 substeps apart): particles whose
    stencil leaves their block's tile take the direct paths, and particles that leave the blocks
    around it trigger an early re-sort; the result equals the in-place substeps."""
    rng = np.random.default_rng(5)
    n_, res, dt, g, steps = 6000, 64, 2e-4, -9.8, 40
    x = rng.uniform(-0.08, 0.08, (n_, 3)) + 0.5
    v = np.tile([[30.0, -20.0, 15.0]], (n_, 1)) + rng.normal(0, 0.5, (n_, 3))  # ~0.4 cells per substep
    vol = 0.16 ** 3 / n_
    E_, nu = 2e3, 0.3
    mu, lam = E_ / (2 * (1 + nu)), E_ * nu / ((1 + nu) * (1 - 2 * nu))
    solver = MPMSolver(torch.tensor(x), res=res, dt=dt, gravity=g, volume=vol, mass=vol, mu_0=mu, lambda_0=lam,
                       v=torch.tensor(v), dtype=dtype, sort_every=25)
    solver.step(steps, check=True)
    got = solver.state()
    ps = ParticleSet(t(x, dtype), t(np.full(n_, vol), dtype), t(np.full(n_, mu), dtype), t(np.full(n_, lam), dtype))
    vv, F, C, Jp = mls_mpm.make_mls_mpm_coefficients(n_, 3, dtype=dtype)
    vv.copy_(t(v, dtype))
    for _ in range(steps):
        mls_mpm.solve_mls_mpm_3d(res, float(res), 1.0, 1 / res, dt, vol, g, ps, vv, F, C, Jp)
    rel = 1e-12 if dtype == torch.float64 else 1e-5
    close(n(got["x"]), n(ps.pos), rel, scale=1.0, what="x")
    close(n(got["v"]), n(vv), 50 * rel, scale=float(np.abs(v).max()), what="v")
    close(n(got["F"]), n(F), 10 * rel, scale=1.0, what="F")
    moved = np.abs(n(got["x"]) - x).max()
    assert moved * res > 12  # more than a block of 8 cells, ~10 cells between scheduled re-sorts


def _fast_cluster(dim, n_, res, dt, cells_per_substep):
    rng = np.random.default_rng(11)
    centre = [0.2, 0.5, 0.45][:dim]
    x = rng.uniform(-0.03, 0.03, (n_, dim)) + centre
    v = np.zeros((n_, dim))
    v[:, 0] = cells_per_substep / res / dt
    v[:, -1] += 0.4 / res / dt
    vol = 0.06 ** dim / n_
    E_, nu = 1e3, 0.3
    return x, v, vol, E_ / (2 * (1 + nu)), E_ * nu / ((1 + nu) * (1 - 2 * nu))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_cluster_at_the_velocity_clamp(dtype):
    """A 3D cluster launched at 2.5 cells per substep: the grid clamps every node velocity to
    0.9 dx / dt (three_d/grid_op.py:25), so it crosses ~11 cells in 12 substeps with no scheduled
    re-sort: its particles leave their chunk blocks' tiles (direct global adds and gathers) and
    then the blocks the plan touches (the fused kernel adds those blocks to the touched list).
    The result equals the in-place substeps."""
    n_, res, dt, g, steps = 3000, 64, 2e-4, -9.8, 12
    x, v, vol, mu, lam = _fast_cluster(3, n_, res, dt, 2.5)
    solver = MPMSolver(torch.tensor(x), res=res, dt=dt, gravity=g, volume=vol, mass=vol, mu_0=mu, lambda_0=lam,
                       v=torch.tensor(v), dtype=dtype, sort_every=64)
    solver.step(steps, check=True)
    got = solver.state()
    ps = ParticleSet(t(x, dtype), t(np.full(n_, vol), dtype), t(np.full(n_, mu), dtype), t(np.full(n_, lam), dtype))
    vv, F, C, Jp = mls_mpm.make_mls_mpm_coefficients(n_, 3, dtype=dtype)
    vv.copy_(t(v, dtype))
    for _ in range(steps):
        mls_mpm.solve_mls_mpm_3d(res, float(res), 1.0, 1 / res, dt, vol, g, ps, vv, F, C, Jp)
    rel = 1e-12 if dtype == torch.float64 else 1e-5
    close(n(got["x"]), n(ps.pos), rel, scale=1.0, what="x")
    close(n(got["v"]), n(vv), 50 * rel, scale=float(np.abs(v).max()), what="v")
    close(n(got["F"]), n(F), 10 * rel, scale=1.0, what="F")
    assert (n(got["x"])[:, 0] - x[:, 0]).min() * res > 10.0


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_2d_cluster_faster_than_two_cells_per_substep(dtype):
    """A 2D cluster at 2.5 cells per substep (the 2D grid rule has no velocity clamp,
    two_d/grid_op.py) with no scheduled re-sort: its particles leave the blocks their plan touches
    within a few substeps, and the fused kernel adds the blocks they reach to the touched list.
    Positions and velocities equal the in-place substeps."""
    from femflow_gb300.solvers.mpm import two_d

    n_, res, dt, g, steps = 3000, 64, 2e-4, -9.8, 12
    x, v, vol, mu, lam = _fast_cluster(2, n_, res, dt, 2.5)
    solver = MPMSolver(torch.tensor(x), res=res, dt=dt, gravity=g, volume=vol, mass=vol, mu_0=mu, lambda_0=lam,
                       v=torch.tensor(v), dtype=dtype, sort_every=64)
    solver.step(steps, check=True)
    got = solver.state()
    gx, gv = t(x, dtype), t(v, dtype)
    gF, gC, gJ = t(np.tile(np.eye(2), (n_, 1, 1)), dtype), t(np.zeros((n_, 2, 2)), dtype), t(np.ones((n_, 1)), dtype)
    for _ in range(steps):
        two_d.solve_mls_mpm_2d(res, float(res), 1.0, mu, lam, vol, 1 / res, dt, vol, g, gx, gv, gF, gC, gJ)
    rel = 1e-12 if dtype == torch.float64 else 1e-5
    close(n(got["x"]), n(gx), rel, scale=1.0, what="x")
    close(n(got["v"]), n(gv), 50 * rel, scale=float(np.abs(v).max()), what="v")
    assert (n(got["x"])[:, 0] - x[:, 0]).min() * res > 2.4 * steps


@pytest.mark.parametrize("variant", [0, 4])
def test_fused_and_separate_launches(variant):
    """Which kernels a sorted run launches: by default P2G once, then the fused G2P + P2G, and a
    plain G2P for the last substep; with variant 4 a P2G and a G2P every substep."""
    s = _scene(torch.float32)
    solver = MPMSolver(torch.tensor(s["x"]), res=s["res"], dt=2e-4, gravity=-9.8, volume=s["vol"],
                       mass=torch.tensor(s["mass"]), mu_0=torch.tensor(s["mu"]), lambda_0=torch.tensor(s["lam"]),
                       v=torch.tensor(s["v"]), dtype=torch.float32, variant=variant)
    prof = solver.profile(6)
    launches = {k: v[1] for k, v in prof.items()}
    if variant == 0:
        assert (launches["p2g"], launches["g2p2g"], launches["g2p"]) == (1, 5, 1)
    else:
        assert (launches["p2g"], launches["g2p2g"], launches["g2p"]) == (6, 0, 6)
    assert launches["grid_update"] == 6
    solver.check()


def test_graph_replay_matches_direct_launches():
    s = _scene(torch.float64)
    kw = dict(res=s["res"], dt=2e-4, gravity=-9.8, volume=s["vol"], mass=torch.tensor(s["mass"]),
              mu_0=torch.tensor(s["mu"]), lambda_0=torch.tensor(s["lam"]), v=torch.tensor(s["v"]),
              dtype=torch.float64)
    a = MPMSolver(torch.tensor(s["x"]), **kw)
    b = MPMSolver(torch.tensor(s["x"]), **kw)
    a.capture(4)  # runs 2 direct warm-up substeps before capturing
    a.step(8)
    b.step(10)
    close(n(a.state()["x"]), n(b.state()["x"]), 1e-12, scale=1.0, what="x graph vs direct")
    a.check()


def test_fp64_diagnostics_match_numpy():
    s = _scene(torch.float32, n_per=1000)
    solver = MPMSolver(torch.tensor(s["x"]), res=s["res"], dt=2e-4, gravity=-9.8, volume=s["vol"],
                       mass=torch.tensor(s["mass"]), mu_0=torch.tensor(s["mu"]), lambda_0=torch.tensor(s["lam"]),
                       v=torch.tensor(s["v"]), dtype=torch.float32)
    solver.step(6)
    d = solver.diagnostics()
    st = solver.sorted_state()
    m = st["mass"].double().cpu().numpy()
    vv = st["v"].double().cpu().numpy()
    xx = st["x"].double().cpu().numpy()
    F = st["F"].double().cpu().numpy()
    assert np.isclose(d["kinetic"], 0.5 * (m * (vv ** 2).sum(1)).sum(), rtol=1e-12)
    assert np.allclose(d["momentum"], (m[:, None] * vv).sum(0), rtol=1e-12, atol=1e-15)
    assert np.isclose(d["mass"], m.sum(), rtol=1e-12)
    assert np.isclose(d["gravitational"], (9.8 * m * xx[:, 1]).sum(), rtol=1e-12)
    assert np.isclose(d["min_det_F"], np.linalg.det(F).min(), rtol=1e-9)
    U, sig, Vt = np.linalg.svd(F)
    R = U @ Vt
    mu = st["mu_0"].double().cpu().numpy(); lam = st["lambda_0"].double().cpu().numpy()
    J = np.linalg.det(F)
    el = (s["vol"] * (mu * ((F - R) ** 2).sum((1, 2)) + 0.5 * lam * (J - 1) ** 2)).sum()
    assert np.isclose(d["elastic"], el, rtol=1e-8)


def test_float32_positions_within_1e_4_of_float64_after_1000_substeps():
    """The accuracy target of the float32 path: the two-cube scene (2 x 32,768 particles, 64^3,
    dt 5e-5, elastic CFL 0.25) run 1000 substeps in float32 and float64 through the resident
    solver; the largest position difference stays below 1e-4 of the domain."""
    from femflow_gb300.scenes import two_cubes

    s = two_cubes(32768)
    kw = dict(res=64, dt=5e-5, gravity=-9.8, volume=s["vol"], mass=s["mass"], mu_0=s["mu"], lambda_0=s["lam"],
              v=torch.tensor(s["v"]))
    a32 = MPMSolver(torch.tensor(s["x"]), dtype=torch.float32, **kw)
    a64 = MPMSolver(torch.tensor(s["x"]), dtype=torch.float64, **kw)
    a32.step(1000, check=True)
    a64.step(1000, check=True)
    err = (a32.positions().double() - a64.positions()).abs().max().item()
    assert err < 1e-4, err


@pytest.mark.parametrize("n_", [1, 2, 255, 256, 257, 511, 512, 513, 1025])
def test_ragged_particle_counts(n_):
    """Particle counts around the chunk size (512 = two particles per thread of a 256-thread CTA)
    through the resident solver (fused G2P + P2G, re-sort every 3 substeps) against the in-place
    substeps, float64."""
    rng = np.random.default_rng(n_)
    res, dt, g, steps = 16, 2e-4, -9.8, 7
    x = rng.uniform(0.3, 0.7, (n_, 3))
    v = rng.normal(0, 0.5, (n_, 3))
    vol = 1e-5
    mu, lam = 300.0, 500.0
    solver = MPMSolver(torch.tensor(x), res=res, dt=dt, gravity=g, volume=vol, mass=vol, mu_0=mu, lambda_0=lam,
                       v=torch.tensor(v), dtype=torch.float64, sort_every=3)
    solver.step(steps, check=True)
    got = solver.state()
    dt64 = torch.float64
    ps = ParticleSet(t(x, dt64), t(np.full(n_, vol), dt64), t(np.full(n_, mu), dt64), t(np.full(n_, lam), dt64))
    vv, F, C, Jp = mls_mpm.make_mls_mpm_coefficients(n_, 3, dtype=dt64)
    vv.copy_(t(v, dt64))
    for _ in range(steps):
        mls_mpm.solve_mls_mpm_3d(res, float(res), 1.0, 1 / res, dt, vol, g, ps, vv, F, C, Jp)
    close(n(got["x"]), n(ps.pos), 1e-12, scale=1.0, what="x")
    close(n(got["v"]), n(vv), 1e-10, scale=max(float(np.abs(v).max()), 1.0), what="v")
    close(n(got["F"]), n(F), 1e-11, scale=1.0, what="F")
    close(n(got["C"]), n(C), 1e-9, scale=max(float(np.abs(n(C)).max()), 1.0), what="C")
