"""The substep on particle arrays in host memory (ffmpm_substep_host), against the oracle.

A caller of solve_mls_mpm_3d (mls_mpm.py:40-79) that keeps its particles in host memory pays for
the copies to the GPU and back on every substep.  With pinned arrays the library copies them in
chunks and overlaps the copies with the kernels: each chunk is scattered, in the caller's order,
as soon as it has landed, and each chunk is gathered and sent back while the next one is
gathered.  These tests hold that path to the float64 oracle (oracle/mpm_oracle.c restating
three_d/*.py and two_d/*.py), to the reference's golden vectors, and to the device-array path.
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle as O
from golden_cases import load, names
from gpu_helpers import TOL, close, n, sign_align
from femflow_gb300 import _native as N
from femflow_gb300 import engine as E
from femflow_gb300.solvers.mpm import mls_mpm
from femflow_gb300.solvers.mpm.particle import ParticleSet
from test_gpu_parity_3d import two_cubes

pytestmark = pytest.mark.gpu
DTYPES = [torch.float64, torch.float32]


def pinned(a, dtype):
    return torch.tensor(np.asarray(a), dtype=dtype).pin_memory()


def _scene(n_per, res, dtype, seed=0):
    s = two_cubes(n_per, res, seed=seed)
    N_ = len(s["x"])
    ps = ParticleSet(pinned(s["x"], dtype), pinned(s["mass"], dtype), pinned(s["mu"], dtype), pinned(s["lam"], dtype))
    state = [pinned(s["v"], dtype), pinned(np.tile(np.eye(3), (N_, 1, 1)), dtype),
             pinned(np.zeros((N_, 3, 3)), dtype), pinned(np.ones((N_, 1)), dtype)]
    return s, ps, state


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("name", names("ref3d_"))
def test_host_substep_matches_reference_golden_vectors(name, dtype):
    d = load(name)
    res, dx, inv_dx, dt, grav, vol, h, steps = d["params"]
    res, steps = int(res), int(steps)
    ps = ParticleSet(pinned(d["x0"], dtype), pinned(d["mass"], dtype), pinned(d["mu0"], dtype),
                     pinned(d["lam0"], dtype))
    v, F, C, Jp = (pinned(d[k + "0"], dtype) for k in ("v", "F", "C", "Jp"))
    assert mls_mpm.P.pinned_host(ps.pos, ps.mass, ps.mu_0, ps.lambda_0, v, F, C, Jp)
    for _ in range(steps):
        mls_mpm.solve_mls_mpm_3d(res, inv_dx, h, dx, dt, vol, grav, ps, v, F, C, Jp)
    tol = TOL[dtype]
    vs = np.abs(d["v"]).max() + abs(grav * dt)
    close(n(ps.pos), d["x"], 5 * tol["x"], scale=1.0, what="x")
    close(n(v), d["v"], 5 * tol["v"], scale=vs, what="v")
    close(n(C), d["C"], 5 * tol["C"], scale=vs * inv_dx, what="C")
    close(n(F), d["F"], 5 * tol["F"], scale=1.0, what="F")


@pytest.mark.parametrize("dtype", DTYPES)
def test_host_substep_two_cubes_against_oracle(dtype):
    """The collision scene, 2 x 2,500 particles, 12 substeps (one chunk)."""
    s, ps, (v, F, C, Jp) = _scene(2500, 32, dtype)
    res, dt, g, steps = s["res"], 2e-4, -9.8, 12
    N_ = len(s["x"])
    x, vo = s["x"].copy(), s["v"].copy()
    Fo, Co, Jo = np.tile(np.eye(3), (N_, 1, 1)), np.zeros((N_, 3, 3)), np.ones((N_, 1))
    for _ in range(steps):
        mls_mpm.solve_mls_mpm_3d(res, float(res), 1.0, 1 / res, dt, s["vol"], g, ps, v, F, C, Jp)
        O.substep_3d(res, float(res), 1.0, 1 / res, dt, s["vol"], g, x, s["mass"], s["mu"], s["lam"], vo, Fo, Co, Jo)
    tol = TOL[dtype]
    close(n(ps.pos), x, 5 * tol["x"], scale=1.0, what="x")
    close(n(v), vo, 5 * tol["v"], scale=np.abs(vo).max(), what="v")
    close(n(F), Fo, 5 * tol["F"], scale=1.0, what="F")


def test_host_substep_equals_device_path_over_chunks():
    """600,000 particles (eight chunks of the pipeline, uneven), float64: the host-array substep and
    the device-array substep agree to rounding of the node sums after 3 substeps."""
    s, ps, (v, F, C, Jp) = _scene(300_000, 64, torch.float64, seed=3)
    res, dt, g = 64, 1e-4, -9.8
    dev = [t.cuda() for t in (ps.pos, ps.mass, ps.mu_0, ps.lambda_0, v, F, C, Jp)]
    pd = ParticleSet(*dev[:4])
    for _ in range(3):
        mls_mpm.solve_mls_mpm_3d(res, float(res), 1.0, 1 / res, dt, s["vol"], g, ps, v, F, C, Jp)
        mls_mpm.solve_mls_mpm_3d(res, float(res), 1.0, 1 / res, dt, s["vol"], g, pd, *dev[4:])
    close(n(ps.pos), n(pd.pos), 1e-13, scale=1.0, what="x")
    close(n(v), n(dev[4]), 1e-11, scale=1.0, what="v")
    close(n(F), n(dev[5]), 1e-12, scale=1.0, what="F")


def test_host_substep_deterministic_mode_is_the_device_path():
    s, ps, (v, F, C, Jp) = _scene(3000, 32, torch.float32, seed=4)
    res, dt, g = 32, 2e-4, -9.8
    dev = [t.cuda() for t in (ps.pos, ps.mass, ps.mu_0, ps.lambda_0, v, F, C, Jp)]
    pd = ParticleSet(*dev[:4])
    for _ in range(4):
        mls_mpm.solve_mls_mpm_3d(res, float(res), 1.0, 1 / res, dt, s["vol"], g, ps, v, F, C, Jp, deterministic=True)
        mls_mpm.solve_mls_mpm_3d(res, float(res), 1.0, 1 / res, dt, s["vol"], g, pd, *dev[4:], deterministic=True)
    assert torch.equal(ps.pos, pd.pos.cpu()) and torch.equal(F, dev[5].cpu())


def test_host_substep_raises_on_a_particle_out_of_the_grid():
    s, ps, (v, F, C, Jp) = _scene(500, 24, torch.float32, seed=5)
    ps.pos[17] = torch.tensor([1.5, 0.5, 0.5])
    with pytest.raises(RuntimeError, match="out of grid"):
        mls_mpm.solve_mls_mpm_3d(24, 24.0, 1.0, 1 / 24, 1e-4, s["vol"], -9.8, ps, v, F, C, Jp)


@pytest.mark.parametrize("dtype", DTYPES)
def test_host_substep_2d_through_the_c_abi(dtype):
    """two_d p2g -> grid_op -> g2p on host arrays with scalar material (two_d/p2g.py:11-29), against
    the oracle's 2D substep (F up to the sign of the reference's SVD rebuild)."""
    d = load("ref2d_c1_small")
    res, dx, inv_dx, dt, grav, vol, mass, mu, lam, h, steps = d["params"]
    res, steps = int(res), int(steps)
    x, v, F, C, Jp = (pinned(d[k + "0"], dtype) for k in ("x", "v", "F", "C", "Jp"))
    dev = [torch.empty_like(a, device="cuda") for a in (x, v, F, C, Jp)]
    prm = E.make_params(2, res, dtype, dx, inv_dx, dt, grav, vol, h, mass, mu, lam)
    host = E.particles_struct(x, v, F, C, Jp)
    ds = E.particles_struct(*dev)
    ws = E.workspace_for(prm, x.shape[0], torch.device("cuda"))
    for _ in range(steps):
        N.call("ffmpm_substep_host", ctypes.byref(prm), ctypes.byref(host), ctypes.byref(ds), ctypes.c_void_p(ws.ptr),
               ctypes.c_size_t(ws.bytes), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    ws.raise_on_status()
    xo, vo, Fo, Co, Jo = (np.array(d[k + "0"], dtype=np.float64) for k in ("x", "v", "F", "C", "Jp"))
    for _ in range(steps):
        O.substep_2d(res, inv_dx, h, mu, lam, mass, dx, dt, vol, grav, xo, vo, Fo, Co, Jo)
    tol = TOL[dtype]
    close(n(x), xo, 5 * tol["x"], scale=1.0, what="x")
    close(n(v), vo, 5 * tol["v"], scale=np.abs(vo).max() + abs(grav * dt), what="v")
    close(sign_align(n(F), Fo), Fo, 5 * tol["F"], scale=1.0, what="F")


def test_host_substep_3d_snow_sends_jp_both_ways():
    """Snow on host arrays (hardening from Jp in P2G, the singular-value clamp and the Jp update in
    G2P, three_d/p2g.py:57-61 and g2p.py:48-58): Jp goes up and comes back every substep, and the
    result matches the oracle's snow substep; the elastic model leaves the host Jp untouched."""
    s = two_cubes(1500, 24, seed=6)
    res, dt, g, h = 24, 1e-4, -9.8, 10.0
    N_ = len(s["x"])
    rng = np.random.default_rng(6)
    F0 = np.tile(np.eye(3), (N_, 1, 1)) + rng.normal(0, 0.02, (N_, 3, 3))
    Jp0 = rng.uniform(0.9, 1.1, (N_, 1))
    for model in ("snow", "neo_hookean"):
        x, v, F, C, Jp = (pinned(a, torch.float64) for a in (s["x"], s["v"], F0, np.zeros((N_, 3, 3)), Jp0))
        mass, mu, lam = (pinned(s[k], torch.float64) for k in ("mass", "mu", "lam"))
        dev = [torch.empty_like(a, device="cuda") for a in (x, v, F, C, Jp, mass, mu, lam)]
        prm = E.make_params(3, res, torch.float64, 1 / res, float(res), dt, g, s["vol"], h, model=model)
        host = E.particles_struct(x, v, F, C, Jp, mass, mu, lam)
        ds = E.particles_struct(*dev)
        ws = E.workspace_for(prm, N_, torch.device("cuda"))
        for _ in range(3):
            N.call("ffmpm_substep_host", ctypes.byref(prm), ctypes.byref(host), ctypes.byref(ds),
                   ctypes.c_void_p(ws.ptr), ctypes.c_size_t(ws.bytes),
                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        ws.raise_on_status()
        xo, vo, Fo, Co, Jo = s["x"].copy(), s["v"].copy(), F0.copy(), np.zeros((N_, 3, 3)), Jp0.copy()
        for _ in range(3):
            O.substep_3d(res, float(res), h, 1 / res, dt, s["vol"], g, xo, s["mass"].copy(), s["mu"].copy(),
                         s["lam"].copy(), vo, Fo, Co, Jo, model=model)
        tol = TOL[torch.float64]
        close(n(x), xo, 5 * tol["x"], scale=1.0, what=f"{model} x")
        close(n(F), Fo, 20 * tol["F"], scale=1.0, what=f"{model} F")
        if model == "snow":
            assert np.abs(Jo - Jp0).max() > 1e-6  # the clamp moved some Jp
            close(n(Jp), Jo, 20 * tol["F"], scale=1.0, what="snow Jp")
        else:
            assert np.array_equal(n(Jp), Jp0)
