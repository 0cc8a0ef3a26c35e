"""Batched 2D scenes (one persistent launch per call) against the oracle and the single-scene path."""
import numpy as np
import pytest
import torch

import oracle as O
from gpu_helpers import TOL, close, n, sign_align, t
from femflow_gb300.batched import Batch2D, random_scenes
from femflow_gb300.solvers.mpm import two_d

pytestmark = pytest.mark.gpu


def small_batch(seed=1):
    sc = random_scenes(7, seed=seed, n_range=(300, 3000), res_range=(24, 96), E_range=(5e2, 5e3))
    sc[3]["model"] = "snow"
    sc[3]["hardening"] = 10.0
    sc[5]["wall_mode"] = "sticky3"
    for s in sc:  # some motion so C and F evolve
        rng = np.random.default_rng(len(s["x"]))
        s["v"] = rng.normal(0, 0.3, size=(len(s["x"]), 2))
    return sc


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_batch_matches_oracle_per_scene(dtype):
    sc = small_batch()
    b = Batch2D(sc, dtype=dtype)
    steps = 5
    b.step(steps)
    assert b.status() == 0
    tol = TOL[dtype]
    for i, s in enumerate(sc):
        if s.get("wall_mode", "reference") != "reference":
            continue  # the oracle implements the reference walls only
        x = s["x"].copy(); v = s["v"].copy(); N_ = len(x)
        F = np.tile(np.eye(2), (N_, 1, 1)); C = np.zeros((N_, 2, 2)); Jp = np.ones((N_, 1))
        for _ in range(steps):
            O.substep_2d(s["res"], float(s["res"]), s.get("hardening", 1.0), s["mu_0"], s["lambda_0"], s["mass"],
                         1.0 / s["res"], s["dt"], s["volume"], -9.8, x, v, F, C, Jp, s.get("model", "neo_hookean"))
        st = b.scene_state(i)
        close(n(st["x"]), x, 5 * tol["x"], scale=1.0, what=f"scene {i} x")
        close(n(st["v"]), v, 5 * tol["v"], scale=np.abs(v).max(), what=f"scene {i} v")
        close(sign_align(n(st["F"]), F), F, 10 * tol["F"], scale=1.0, what=f"scene {i} F")


def test_batch_matches_single_scene_path_with_sticky_walls():
    sc = small_batch(seed=2)
    b = Batch2D(sc, dtype=torch.float64)
    b.step(4)
    for i in (5,):
        s = sc[i]
        dtype = torch.float64
        x, v = t(s["x"], dtype), t(s["v"], dtype)
        N_ = x.shape[0]
        F = torch.eye(2, dtype=dtype, device="cuda").repeat(N_, 1, 1).contiguous()
        C = torch.zeros((N_, 2, 2), dtype=dtype, device="cuda")
        Jp = torch.ones((N_, 1), dtype=dtype, device="cuda")
        for _ in range(4):
            two_d.solve_mls_mpm_2d(s["res"], float(s["res"]), 1.0, s["mu_0"], s["lambda_0"], s["mass"], 1.0 / s["res"],
                                   s["dt"], s["volume"], -9.8, x, v, F, C, Jp, wall_mode="sticky3")
        st = b.scene_state(i)
        close(n(st["x"]), n(x), 1e-12, scale=1.0, what="x sticky3")


def test_batch_graph_replay_and_autotune():
    sc = small_batch(seed=3)
    a = Batch2D(sc, dtype=torch.float64)
    c = Batch2D(sc, dtype=torch.float64)
    best, timings = a.autotune(steps=1)  # advances a by 1 substep per candidate tried
    assert best in [(128, 0), (256, 0), (512, 0), (256, 2), (512, 1)]
    used = len(timings) * 2 if timings else 0  # time_call: 1 warm-up + 3 timed launches of `steps`
    a2 = Batch2D(sc, dtype=torch.float64)
    a2.capture(4)  # one direct substep before capturing
    a2.step(8)
    c.step(9)
    close(n(a2.scene_state(2)["x"]), n(c.scene_state(2)["x"]), 1e-12, scale=1.0, what="graph vs direct")
    assert a.status() == 0 and a2.status() == 0


def test_batch_256_scenes_graph_against_oracle():
    """The batched workload at full scale: 256 seeded scenes (2k-64k particles each, grids 64^2 to
    256^2, the stable variant of E), autotuned launch shape, one 100-substep CUDA graph; a seeded
    sample of scenes against the oracle's 2D substep after the 100 substeps."""
    from femflow_gb300.batched import stable_variant

    sc = stable_variant(random_scenes(256, seed=0))
    b = Batch2D(sc, dtype=torch.float32)
    b.autotune(steps=1)  # advances every scene by the substeps used for timing
    b.reset()  # zero the grids and the status; the particle state keeps the autotuning substeps
    start = [b.scene_state(i) for i in range(len(sc))]
    b.capture(100)  # one direct substep before the capture
    b.step(100)
    assert b.status() == 0
    rng = np.random.default_rng(7)
    sample = sorted(rng.choice(len(sc), size=5, replace=False, p=None))
    for i in sample:
        s, st0 = sc[i], start[i]
        x, v = n(st0["x"]), n(st0["v"])
        F, C, Jp = n(st0["F"]), n(st0["C"]), n(st0["Jp"]).reshape(-1, 1)
        for _ in range(101):
            O.substep_2d(s["res"], float(s["res"]), 1.0, s["mu_0"], s["lambda_0"], s["mass"], 1.0 / s["res"], s["dt"],
                         s["volume"], -9.8, x, v, F, C, Jp)
        got = b.scene_state(i)
        close(n(got["x"]), x, 1e-5, scale=1.0, what=f"scene {i} x")
        close(n(got["v"]), v, 1e-3, scale=max(np.abs(v).max(), 1e-3), what=f"scene {i} v")


def test_one_call_of_many_substeps_equals_single_substep_calls():
    """A call of k substeps fuses each substep's G2P with the next P2G and visits only each scene's
    box of touched nodes; k calls of one substep do neither across calls.  Both give the same
    state (float64: only the order of the atomic sums differs), in the caller's particle order."""
    sc = small_batch(seed=5)
    a = Batch2D(sc, dtype=torch.float64)
    c = Batch2D(sc, dtype=torch.float64)
    a.step(7)
    for _ in range(7):
        c.step(1)
    assert a.status() == 0 and c.status() == 0
    for i in range(len(sc)):
        sa, sb = a.scene_state(i), c.scene_state(i)
        for k in ("x", "v", "F", "C", "Jp"):
            close(n(sa[k]), n(sb[k]), 1e-10, scale=max(float(np.abs(n(sb[k])).max()), 1.0), what=f"scene {i} {k}")


def test_batch_orders_particles_by_cell_and_maps_back():
    sc = small_batch(seed=6)
    b = Batch2D(sc, dtype=torch.float64)
    for i, s in enumerate(sc):
        np.testing.assert_array_equal(n(b.scene_state(i)["x"]), s["x"])
        np.testing.assert_array_equal(n(b.scene_state(i)["v"]), s["v"])
        a0, a1 = int(b.offsets[i]), int(b.offsets[i + 1])
        xs = n(b.x[:, a0:a1].T)
        cell = np.floor(xs * s["res"] - 0.5).astype(np.int64)
        key = cell[:, 0] * (s["res"] + 2) + cell[:, 1]
        assert (np.diff(key) >= 0).all()
        k = 17 % len(s["x"])
        np.testing.assert_array_equal(n(b.x[:, b.position(i, k)]), s["x"][k])


def test_batch_with_an_empty_scene():
    """A scene without particles (zero-count entries in the particle offsets, an empty node box)
    between scenes that have them: the others still match the oracle."""
    sc = small_batch(seed=8)[:4]
    empty = dict(sc[1])
    empty["x"] = np.zeros((0, 2))
    empty["v"] = np.zeros((0, 2))
    sc = [sc[0], empty, sc[2], sc[3]]
    b = Batch2D(sc, dtype=torch.float64)
    b.step(3)
    assert b.status() == 0
    assert b.scene_state(1)["x"].shape == (0, 2)
    for i in (0, 2, 3):
        s = sc[i]
        if s.get("wall_mode", "reference") != "reference":
            continue
        x = s["x"].copy(); v = s["v"].copy(); N_ = len(x)
        F = np.tile(np.eye(2), (N_, 1, 1)); C = np.zeros((N_, 2, 2)); Jp = np.ones((N_, 1))
        for _ in range(3):
            O.substep_2d(s["res"], float(s["res"]), s.get("hardening", 1.0), s["mu_0"], s["lambda_0"], s["mass"],
                         1.0 / s["res"], s["dt"], s["volume"], -9.8, x, v, F, C, Jp, s.get("model", "neo_hookean"))
        close(n(b.scene_state(i)["x"]), x, 5 * TOL[torch.float64]["x"], scale=1.0, what=f"scene {i} x")
