"""Failure detection on the GPU: every failure is made on the host and read back as a status bit.

* A NaN planted in F (host side) must raise FFMPM_STATUS_NONFINITE (and a RuntimeError through
  the Python mirror), in 3D, in 2D and in a batch.  The reference's only detector is the
  out-of-grid check (utils.py:138-150); a NaN that stays inside the grid passes it silently.
* The bounded waits must end and report FFMPM_STATUS_TIMEOUT when what they wait for never comes.
  The injection bits make one wait impossible to satisfy (the first radix tile never publishes its
  digit counts; one CTA of the batched launch never reaches the grid barrier), and a small wait
  limit makes the give-up quick.  Afterwards the same context must sort and step correctly again.
No kernel is made to fault, trap or hang: every wait here is bounded and every index stays in range.
"""
import ctypes

import numpy as np
import pytest
import torch

from gpu_helpers import close, n
from femflow_gb300 import _native as N
from femflow_gb300 import engine as E
from femflow_gb300.batched import Batch2D, random_scenes
from femflow_gb300.solver import MPMSolver
from femflow_gb300.solvers.mpm import mls_mpm
from femflow_gb300.solvers.mpm.particle import ParticleSet
from test_gpu_parity_3d import two_cubes
from test_gpu_sort_and_solver import host_keys

pytestmark = pytest.mark.gpu


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _solver(dim, sort_every=8, n_per=4000):
    rng = np.random.default_rng(5)
    x = rng.uniform(0.3, 0.5, size=(2 * n_per, dim))
    E_, nu = 3e3, 0.3
    mu, lam = E_ / (2 * (1 + nu)), E_ * nu / ((1 + nu) * (1 - 2 * nu))
    vol = 0.2 ** dim / len(x)
    return MPMSolver(torch.tensor(x), res=48, dt=1e-4, volume=vol, mass=vol, mu_0=mu, lambda_0=lam,
                     sort_every=sort_every)


@pytest.mark.parametrize("dim,sort_every", [(3, 8), (3, 1), (2, 8)])
def test_nan_in_F_raises_nonfinite(dim, sort_every):
    s = _solver(dim, sort_every)
    s.step(2, check=True)  # a clean start
    s._cur.F[0, 123] = float("nan")  # plant a NaN in one particle's F on the host side of the ABI
    s.step(2)
    st, _ = s.status()
    assert st & N.STATUS_NONFINITE, st
    with pytest.raises(RuntimeError, match="non-finite"):
        s.check()


def test_nan_in_F_through_the_reference_api():
    sc = two_cubes(500, 24)
    dev = "cuda"
    x = torch.tensor(sc["x"], dtype=torch.float32, device=dev)
    nn = x.shape[0]
    ps = ParticleSet(x, torch.tensor(sc["mass"], dtype=torch.float32, device=dev),
                     torch.tensor(sc["mu"], dtype=torch.float32, device=dev),
                     torch.tensor(sc["lam"], dtype=torch.float32, device=dev))
    v = torch.tensor(sc["v"], dtype=torch.float32, device=dev)
    F = torch.eye(3, device=dev).repeat(nn, 1, 1).contiguous()
    C = torch.zeros((nn, 3, 3), device=dev)
    Jp = torch.ones((nn, 1), device=dev)
    F[7, 1, 2] = float("inf")
    with pytest.raises(RuntimeError, match="non-finite"):
        mls_mpm.solve_mls_mpm_3d(sc["res"], float(sc["res"]), 1.0, 1 / sc["res"], 2e-4, sc["vol"], -9.8, ps, v,
                                 F, C, Jp)


def _batch():
    sc = random_scenes(5, seed=4, n_range=(300, 2000), res_range=(24, 64), E_range=(5e2, 3e3))
    for s in sc:
        rng = np.random.default_rng(len(s["x"]))
        s["v"] = rng.normal(0, 0.3, size=(len(s["x"]), 2))
    return sc


def test_nan_in_batched_scene_raises_nonfinite():
    b = Batch2D(_batch(), dtype=torch.float32)
    b.step(1)
    assert b.status() == 0
    a = int(b.offsets[2])
    b.F[3, a + 5] = float("nan")
    b.step(1)
    assert b.status() & N.STATUS_NONFINITE


def _sort(prm, xd, ws):
    nn = xd.shape[0]
    keys = torch.full((nn,), -7, dtype=torch.int32, device="cuda")
    perm = torch.full((nn,), -7, dtype=torch.int32, device="cuda")
    N.call("ffmpm_sort_by_block", ctypes.byref(prm), ctypes.c_void_p(xd.data_ptr()), nn,
           ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(ws.ptr),
           ctypes.c_size_t(ws.bytes), _stream())
    torch.cuda.synchronize()
    return keys.cpu().numpy().view(np.uint32).astype(np.uint64), perm.cpu().numpy().astype(np.int64)


def test_radix_lookback_runs_out_and_the_next_sort_is_exact():
    rng = np.random.default_rng(8)
    nn, res = 300_001, 128  # 74 tiles of 4096 keys per pass
    x = rng.uniform(0.05, 0.95, size=(nn, 3)).astype(np.float32)
    xd = torch.from_numpy(x).cuda()
    stalled = E.make_params(3, res, torch.float32, 1 / res, float(res), 1e-4, wait_limit=256,
                            inject=N.INJECT_LOOKBACK_STALL)
    ws = E.Workspace(stalled, nn, "cuda")
    _sort(stalled, xd, ws)
    st, _ = ws.status()
    assert st & N.STATUS_TIMEOUT, st
    # the context is still usable: clear the word and sort again without the injection
    ws.clear_status()
    clean = E.make_params(3, res, torch.float32, 1 / res, float(res), 1e-4)
    keys, perm = _sort(clean, xd, ws)
    st, _ = ws.status()
    assert st == 0
    hk = host_keys(x, res, 8, False)
    ref = np.argsort(hk, kind="stable")
    assert np.array_equal(keys, hk[ref])
    assert np.array_equal(perm, ref)


def test_static_sort_reports_a_lookback_that_ran_out():
    rng = np.random.default_rng(9)
    nn, res = 200_000, 128
    x = torch.from_numpy(rng.uniform(0.05, 0.95, size=(nn, 3)).astype(np.float32)).cuda()
    status = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    prm = E.make_params(3, res, torch.float32, 1 / res, float(res), 1e-4, wait_limit=256,
                        inject=N.INJECT_LOOKBACK_STALL)
    keys = torch.empty(nn, dtype=torch.int32, device="cuda")
    perm = torch.empty(nn, dtype=torch.int32, device="cuda")
    N.call("ffmpm_sort_by_block_static", ctypes.byref(prm), ctypes.c_void_p(x.data_ptr()), nn,
           ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(status.data_ptr()),
           _stream())
    torch.cuda.synchronize()
    assert int(status.item()) & N.STATUS_TIMEOUT


def test_batched_barrier_runs_out_and_the_batch_recovers():
    sc = _batch()
    b = Batch2D(sc, dtype=torch.float64)
    ref = Batch2D(sc, dtype=torch.float64)
    b.set_waits(wait_limit=2000, inject=N.INJECT_BARRIER_ABSENT)
    # two calls of one launch each: every call starts its barrier count from zero, so in each launch
    # every CTA but the absent one gives up at the first barrier
    b.step(1)
    assert b.status() & N.STATUS_TIMEOUT
    b.step(1)
    assert b.status() & N.STATUS_TIMEOUT
    # no launch got past its first barrier, so no particle moved; after a reset the batch steps
    # exactly like one that never failed
    b.reset()
    assert b.status() == 0
    b.step(3)
    ref.step(3)
    assert b.status() == 0 and ref.status() == 0
    for i in range(len(sc)):
        close(n(b.scene_state(i)["x"]), n(ref.scene_state(i)["x"]), 1e-12, scale=1.0, what=f"scene {i} x")
