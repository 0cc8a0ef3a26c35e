"""The benchmarked solver path against the float64 C oracle, at scale and over long horizons.

The throughput figure times the resident solver: particles kept block-sorted in HBM, a re-sort
every 8 substeps, the fused G2P + next-substep P2G kernel, substeps replayed from a captured
40-substep CUDA graph.  These tests run exactly that configuration (``MPMSolver(sort_every=8)``
+ ``capture(40)``) on the two-cube collision scene and compare it with the oracle's serial float64
restatement of three_d/p2g.py, grid_op.py and g2p.py (oracle/mpm_oracle.c, pinned to the
reference's own outputs by tests/test_oracle_golden.py), so that every re-sort, kept plan and
stray-particle path of the fused kernel is checked against the reference's arithmetic and not
against other code of this repository.
"""
import numpy as np
import pytest
import torch

import oracle as O
from gpu_helpers import close, n
from femflow_gb300.scenes import two_cubes
from femflow_gb300.solver import MPMSolver

pytestmark = pytest.mark.gpu

DT, G = 5e-5, -9.8


def _solver(s, res, dtype):
    return MPMSolver(torch.tensor(s["x"]), res=res, dt=DT, gravity=G, volume=s["vol"], mass=s["mass"],
                     mu_0=s["mu"], lambda_0=s["lam"], v=torch.tensor(s["v"]), dtype=dtype, sort_every=8)


def _oracle(s, res, steps):
    nn = s["n"]
    x, v = s["x"].copy(), s["v"].copy()
    F = np.tile(np.eye(3), (nn, 1, 1))
    C = np.zeros((nn, 3, 3))
    Jp = np.ones((nn, 1))
    m, mu, lam = np.full(nn, s["mass"]), np.full(nn, s["mu"]), np.full(nn, s["lam"])
    for _ in range(steps):
        O.substep_3d(res, float(res), 1.0, 1.0 / res, DT, s["vol"], G, x, m, mu, lam, v, F, C, Jp)
    return dict(x=x, v=v, F=F, C=C)


def _run_graphed(solver, total):
    """``total`` substeps: the capture's own two warm-up substeps, then 40-substep graph replays,
    then the remainder as a direct call."""
    solver.capture(40)
    left = total - solver.steps_done
    solver.step(left // 40 * 40)
    if left % 40:
        solver.step(left % 40)
    solver.check()
    assert solver.steps_done == total
    return solver.state()


# measured on a GB300: float32 x 2.0e-6, v 1.2e-6 (of max |v| 1), F 7.6e-8; float64 x 6.7e-16,
# v 1.2e-13, F 4.6e-15
@pytest.mark.parametrize("dtype,tol", [(torch.float32, dict(x=1e-5, v=2e-5, F=1e-6)),
                                       (torch.float64, dict(x=1e-13, v=1e-11, F=1e-12))])
def test_benchmarked_path_against_oracle_65k_particles_242_substeps(dtype, tol):
    """2 x 32,768 particles on the benchmark's 128^3 grid and dt, 242 substeps (30 re-sorts), in the
    benchmark's configuration, against the oracle."""
    s = two_cubes(32768)
    res, steps = 128, 242
    got = _run_graphed(_solver(s, res, dtype), steps)
    want = _oracle(s, res, steps)
    vmax = float(np.abs(want["v"]).max())
    ex = close(n(got["x"]), want["x"], tol["x"], scale=1.0, what="x")
    ev = close(n(got["v"]), want["v"], tol["v"], scale=vmax, what="v")
    eF = close(n(got["F"]), want["F"], tol["F"], scale=1.0, what="F")
    print(f"{dtype}: max |x - x_oracle| {ex:.2e}, |v - v_oracle| {ev:.2e} (of {vmax:.2f}), |F - F_oracle| {eF:.2e}")


def test_1000_substeps_against_oracle_16k_particles():
    """The accuracy target on the oracle itself: 2 x 8,192 particles, 64^3 grid, 1000 substeps (the
    cubes close the gap between them and meet), benchmark configuration.  float64 on the GPU
    follows the oracle to rounding; float32 stays within 1e-4 of the domain in position."""
    s = two_cubes(8192)
    res, steps = 64, 1000
    want = _oracle(s, res, steps)
    g64 = _run_graphed(_solver(s, res, torch.float64), steps)
    g32 = _run_graphed(_solver(s, res, torch.float32), steps)
    # measured on a GB300: float64 x 1.9e-15, float32 x 5.2e-6
    e64 = close(n(g64["x"]), want["x"], 1e-12, scale=1.0, what="float64 x after 1000 substeps")
    close(n(g64["F"]), want["F"], 1e-11, scale=1.0, what="float64 F after 1000 substeps")
    e32 = close(n(g32["x"]), want["x"], 1e-4, scale=1.0, what="float32 x after 1000 substeps")
    print(f"after 1000 substeps: float64 max |x - x_oracle| {e64:.2e}, float32 {e32:.2e} (domain 1)")
