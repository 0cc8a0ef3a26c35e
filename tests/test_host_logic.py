"""Host-side pieces that need no GPU: parameter packing, particle containers, helpers."""
import ctypes

import numpy as np
import pytest
import torch

from femflow_gb300 import _native as N
from femflow_gb300 import engine as E
from femflow_gb300.solvers.mpm import particle as PT
from femflow_gb300.solvers.mpm import utils as U


def test_abi_struct_sizes():
    """The ctypes mirrors have the sizes the library is compiled against (static_assert in capi.cu)."""
    assert ctypes.sizeof(N.Params) == 504
    assert ctypes.sizeof(N.Particles) == 80


def test_params_packing():
    p = E.make_params(3, 64, torch.float64, 1 / 64, 64.0, 1e-4, -9.8, 2e-6, 1.0, model="snow", wall_mode="sticky3")
    assert (p.dim, p.res, p.real_bytes, p.model, p.wall_mode) == (3, 64, 8, 1, 1)
    assert p.gravity == -9.8 and p.volume == 2e-6
    with pytest.raises(TypeError):
        E.make_params(3, 64, torch.int32, 1, 1, 1)


def test_particle_set_roundtrip():
    ps = [PT.Particle(np.array([0.1, 0.2, 0.3]), 0.0, 2.0, 3.0, 4.0), PT.Particle(np.array([0.4, 0.5, 0.6]), 0.0, 1.0, 1.0, 1.0)]
    s = PT.ParticleSet.from_particles(ps)
    assert s.pos.shape == (2, 3) and s.mass.tolist() == [2.0, 1.0]
    assert s.lambda_0.tolist() == [3.0, 1.0] and s.mu_0.tolist() == [4.0, 1.0]  # Particle(pos, force, mass, lambda_, mu)
    s.pos += 1.0
    s.write_positions(ps)
    assert np.allclose(ps[0].pos, [1.1, 1.2, 1.3])
    np.testing.assert_allclose(PT.map_particles_to_pos(ps, 2.0), np.array([[1.1, 1.2, 1.3], [1.4, 1.5, 1.6]]).reshape(-1) / 2)


def test_particle_set_length_mismatch():
    with pytest.raises(ValueError):
        PT.ParticleSet(torch.zeros(3, 3), torch.zeros(2), torch.zeros(3), torch.zeros(3))


def test_utils_match_reference_formulas():
    assert U.constant_hardening(2.0, 3.0, 10.0) == (20.0, 30.0)
    mu, lam = U.snow_hardening(2.0, 3.0, 10.0, np.array([0.9]))
    assert np.isclose(mu, 2.0 * np.exp(1.0)) and np.isclose(lam, 3.0 * np.exp(1.0))
    assert U.oob(np.array([0, 0, 127]), 129, np.array([0, 0, 2]))
    assert not U.oob(np.array([0, 0, 126]), 129, np.array([0, 0, 2]))
    assert np.isclose(U.Ev_to_mu(1e4, 0.2), 4166.666666666667)
    assert np.isclose(U.Ev_to_lambda(1e4, 0.2), 2777.777777777778)


def test_no_cpu_fallback_without_gpu():
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from femflow_gb300.solvers.mpm import mls_mpm
    v, F, C, Jp = mls_mpm.make_mls_mpm_coefficients(4, 3, device="cpu")
    ps = PT.ParticleSet(torch.rand(4, 3) * 0.5 + 0.25, torch.ones(4), torch.ones(4), torch.ones(4))
    with pytest.raises(RuntimeError, match="CUDA"):
        mls_mpm.solve_mls_mpm_3d(16, 16.0, 1.0, 1 / 16, 1e-4, 1.0, -9.8, ps, v, F, C, Jp)


def test_kernels_per_call():
    """Launch counts of a sorted run (host-only query): fused G2P + P2G by default, separate G2P and
    P2G launches for one substep and variant 4."""

    def count(nsteps, **kw):
        p = E.make_params(3, 128, torch.float32, 1 / 128, 128.0, 1e-4, **kw)
        c = ctypes.c_int64()
        N.call("ffmpm_kernels_per_call", ctypes.byref(p), 1 << 20, int(nsteps), ctypes.byref(c))
        return c.value

    info = (ctypes.c_int64 * 8)()
    N.call("ffmpm_plan_info", ctypes.byref(E.make_params(3, 128, torch.float32, 1 / 128, 128.0, 1e-4)), 1 << 20, info)
    sort = 1 + info[4] + 3  # digit histogram, radix passes, three plan kernels
    every8 = 8 << 8
    # fused: (keys, sort, P2G) + (n - 1) (grid, fused) + the re-sorts at k = 8 + (grid, G2P)
    assert count(10, variant=every8) == (2 + sort) + 9 * 2 + 1 * sort + 2
    assert count(2, variant=every8) == (2 + sort) + 2 + 2
    assert count(20, variant=every8) == (2 + sort) + 19 * 2 + 2 * sort + 2
    # one substep and variant 4: decide, sort, P2G, grid, G2P per substep, keys once
    assert count(1, variant=every8) == 1 + sort + 3 + 1
    assert count(10, variant=every8 | 4) == 10 * (1 + sort + 3) + 1
    assert count(0, variant=every8) == 0


def test_shared_memory_capacity_checks():
    """3D with 16-node block sides: in float32 the fused kernel's two tiles do not fit in shared
    memory, so sorted runs keep separate launches; in float64 not even the cell-run P2G fits, and
    the operations answer FFMPM_ERR_UNSUPPORTED (before any device work)."""
    every8 = 8 << 8

    def params(dtype, bs):
        return E.make_params(3, 128, dtype, 1 / 128, 128.0, 1e-4, block_size=bs, variant=every8)

    def count(prm, nsteps):
        c = ctypes.c_int64()
        N.call("ffmpm_kernels_per_call", ctypes.byref(prm), 1 << 20, int(nsteps), ctypes.byref(c))
        return c.value

    info = (ctypes.c_int64 * 8)()
    N.call("ffmpm_plan_info", ctypes.byref(params(torch.float32, 16)), 1 << 20, info)
    sort = 1 + info[4] + 3
    # block side 16 in float32: separate launches (decide, sort, P2G, grid, G2P per substep, keys once)
    assert count(params(torch.float32, 16), 10) == 10 * (1 + sort + 3) + 1
    # block side 8: the fused kernel
    assert count(params(torch.float32, 8), 10) < 10 * (1 + sort + 3) + 1
    lib = N.load()
    P = N.Particles()
    P.n = 16
    for dtype, want in ((torch.float64, N.ERR_UNSUPPORTED), (torch.float32, N.ERR_WORKSPACE)):
        prm = params(dtype, 16)
        rc = lib.ffmpm_substep(ctypes.byref(prm), ctypes.byref(P), None, ctypes.c_size_t(0), None)
        assert rc == want, (dtype, rc)


def test_particle_count_limit():
    """Workspace calls take fewer than 2^30 particles (the sort's look-back words hold 30-bit counts)."""
    prm = E.make_params(3, 64, torch.float32, 1 / 64, 64.0, 1e-4)
    out = ctypes.c_size_t(0)
    lib = N.load()
    assert lib.ffmpm_workspace_size(ctypes.byref(prm), (1 << 30) - 1, ctypes.byref(out)) == N.OK
    assert lib.ffmpm_workspace_size(ctypes.byref(prm), 1 << 30, ctypes.byref(out)) == N.ERR_BADARG


def test_batch_cell_order_is_a_per_scene_stable_sort_by_base_cell():
    from femflow_gb300.batched import batch_cell_order

    rng = np.random.default_rng(3)
    counts, res = [500, 0, 1300, 7], [32, 64, 128, 16]
    offsets = np.concatenate([[0], np.cumsum(counts)])
    x = rng.uniform(0.1, 0.9, (offsets[-1], 2))
    perm = batch_cell_order(x, offsets, res)
    assert sorted(perm.tolist()) == list(range(offsets[-1]))
    for s, r in enumerate(res):
        a, b = offsets[s], offsets[s + 1]
        p = perm[a:b]
        assert ((p >= a) & (p < b)).all()  # scenes stay in place
        cell = np.floor(x[p] * r - 0.5).astype(np.int64)
        key = cell[:, 0] * (r + 2) + cell[:, 1]
        assert (np.diff(key) >= 0).all()
        same = np.diff(key) == 0
        assert (np.diff(p)[same] > 0).all()  # stable: equal cells keep the caller's order


def test_rollout_cell_order_and_its_inverse():
    import torch
    from femflow_gb300.diff import cell_order

    x = torch.rand(2000, 3, dtype=torch.float64)
    p = cell_order(x, 16)
    inv = torch.empty_like(p)
    inv[p] = torch.arange(len(p))
    assert torch.equal(x[p][inv], x)
    b = (torch.floor(x[p] * 16 - 0.5) + 1).long()
    key = (b[:, 0] * 19 + b[:, 1]) * 19 + b[:, 2]
    assert (key[1:] >= key[:-1]).all()


def test_on_policy_rows_beyond_the_target_bound_are_dropped():
    import torch
    from femflow_gb300.learned_eval import bounded_rows

    X = torch.randn(6, 128).to(torch.bfloat16)
    T = torch.randn(6, 12)
    T[1, 3] = 500.0           # far beyond the bound
    T[4, 0] = float("nan")    # not finite
    X[5, 7] = float("inf")    # feature not finite
    scale = torch.full((12,), 2.0)
    Xk, Tk, dropped = bounded_rows(X, T, scale, 30.0)
    assert dropped == 3 and Xk.shape[0] == 3
    assert torch.equal(Tk, T[[0, 2, 3]])


def test_autotuner_picks_the_fastest_and_caches(tmp_path, monkeypatch):
    from femflow_gb300 import autotune as AT

    fake = {(128, 0): 3.0, (256, 0): 1.0, (512, 0): 2.0}
    ran = []

    def fake_time(fn, iters=3, warmup=1):
        fn()
        return fake[ran[-1]]

    def run(c):
        if c == (1024, 0):
            raise RuntimeError("cannot launch")  # skipped, as a configuration that fails here
        ran.append(c)

    monkeypatch.setattr(AT, "time_call", fake_time)
    monkeypatch.setattr(AT, "_CACHE", {})
    monkeypatch.setenv("FFMPM_TUNE_CACHE", str(tmp_path / "tune.json"))
    cands = [(128, 0), (1024, 0), (256, 0), (512, 0)]
    best, timings = AT.tune(("sig", 1), cands, run)
    assert best == (256, 0) and set(timings) == {(128, 0), (256, 0), (512, 0)}
    # in-process cache: nothing runs again
    ran.clear()
    assert AT.tune(("sig", 1), cands, run) == ((256, 0), {}) and not ran
    # a new process (empty in-process cache) reads the file cache
    monkeypatch.setattr(AT, "_CACHE", {})
    assert AT.tune(("sig", 1), cands, run) == ((256, 0), {}) and not ran
    # no candidate can launch: an error, not a silent default
    with pytest.raises(RuntimeError, match="no candidate"):
        AT.tune(("sig", 2), [(1024, 0)], run)


@pytest.mark.parametrize("dim", [2, 3])
def test_rollout_state_pack_round_trip(dim):
    from femflow_gb300.diff import _rows, pack, unpack

    n = 37
    x, v = torch.randn(n, dim), torch.randn(n, dim)
    F, C = torch.randn(n, dim, dim), torch.randn(n, dim, dim)
    buf = pack(x, v, F, C)
    (ox, ov, oF, oC), rows = _rows(dim)
    assert buf.shape == (rows, n) and rows == 2 * dim + 2 * dim * dim
    assert torch.equal(buf[ox:ov].t(), x) and torch.equal(buf[oC:rows].t().reshape(n, dim, dim), C)
    for a, b in zip(unpack(buf), (x, v, F, C)):
        assert torch.equal(a, b)
