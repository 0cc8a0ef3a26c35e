"""GPU MPMSimulation driver (femflow/simulation/mpm/simulation.py) against the oracle."""
import os

import numpy as np
import pytest

import oracle as O
from femflow_gb300.simulation.mpm.primitives import generate_cube_points
from femflow_gb300.simulation.mpm.simulation import MPMSimulation

pytestmark = pytest.mark.gpu


class _Mesh:
    def __init__(self, v):
        self.vertices = np.asarray(v, dtype=np.float32).reshape(-1)  # viz/mesh.py stores flat float32


def test_simulation_driver_matches_oracle(tmp_path):
    coeff = 0.5
    a = generate_cube_points((0.5, 0.9), (0.6, 1.0), (0.5, 0.9), 12)   # before tightening
    b = generate_cube_points((0.9, 1.3), (0.6, 1.0), (0.9, 1.3), 12)
    params = [(2e-5, 3e3, 0.3), (1e-5, 6e3, 0.25)]
    steps = 8
    sim = MPMSimulation(str(tmp_path / "out"), steps, 1e-4, 2e-5, 1e-5, 1e-5, -9.8, 3e3, 6e3, 0.3, 0.25, 1.0, 32,
                        coeff, save_displacements=True)
    sim.load(meshes=[_Mesh(a), _Mesh(b)], params=params)
    sim.start()
    sim.join(timeout=120)
    assert not sim.running
    assert len(sim.displacements) == steps + 1
    assert len(os.listdir(tmp_path / "out")) == steps + 1
    # oracle with the same particles (float32 vertices, as Mesh stores them) and material
    x = np.concatenate([np.asarray(_Mesh(a).vertices, dtype=np.float64).reshape(-1, 3),
                        np.asarray(_Mesh(b).vertices, dtype=np.float64).reshape(-1, 3)]) * coeff
    n = len(x)
    na = len(a)
    mass = np.r_[np.full(na, params[0][0]), np.full(n - na, params[1][0])]
    mu = np.r_[np.full(na, 3e3 / (2 * 1.3)), np.full(n - na, 6e3 / (2 * 1.25))]
    lam = np.r_[np.full(na, 3e3 * 0.3 / (1.3 * 0.4)), np.full(n - na, 6e3 * 0.25 / (1.25 * 0.5))]
    v = np.zeros((n, 3)); F = np.tile(np.eye(3), (n, 1, 1)); C = np.zeros((n, 3, 3)); Jp = np.ones((n, 1))
    for _ in range(steps):
        O.substep_3d(32, 32.0, 1.0, 1 / 32, 1e-4, 1e-5, -9.8, x, mass, mu, lam, v, F, C, Jp)
    got = sim.displacements[-1].reshape(-1, 3) * coeff
    assert np.abs(got - x).max() < 2e-6
    np.testing.assert_allclose(np.load(tmp_path / "out" / f"{steps}.npy"), sim.displacements[-1])


class _Recording(list):
    """A displacements list that notes how many substeps the solver had been given at each append."""

    def __init__(self, sim, items):
        super().__init__(items)
        self.sim, self.enqueued = sim, []

    def append(self, item):
        self.enqueued.append(self.sim.solver.steps_done)
        super().append(item)


def test_simulation_chunks_graph_and_live_displacements(tmp_path):
    """100 substeps in chunks of 40 (a direct chunk, the captured graph, a remainder of 20) with 4
    pinned host buffers: every substep's displacement equals the oracle's, and displacements are
    appended while later substeps are still being handed to the GPU (as the reference appends after
    each substep, simulation.py:140-142, for its GUI thread to read)."""
    coeff = 0.5
    a = generate_cube_points((0.5, 0.9), (0.6, 1.0), (0.5, 0.9), 12)
    b = generate_cube_points((0.9, 1.3), (0.6, 1.0), (0.9, 1.3), 12)
    params = [(2e-5, 3e3, 0.3), (1e-5, 6e3, 0.25)]
    steps = 100
    sim = MPMSimulation(str(tmp_path / "out"), steps, 1e-4, 2e-5, 1e-5, 1e-5, -9.8, 3e3, 6e3, 0.3, 0.25, 1.0, 32,
                        coeff, save_displacements=True, chunk=40, host_buffers=4)
    sim.load(meshes=[_Mesh(a), _Mesh(b)], params=params)
    sim.displacements = _Recording(sim, sim.displacements)
    sim.start()
    sim.join(timeout=300)
    assert not sim.running
    assert len(sim.displacements) == steps + 1
    # the first displacement arrived before the second chunk was given to the solver
    assert sim.displacements.enqueued[0] < steps, sim.displacements.enqueued[:3]
    x = np.concatenate([np.asarray(_Mesh(a).vertices, dtype=np.float64).reshape(-1, 3),
                        np.asarray(_Mesh(b).vertices, dtype=np.float64).reshape(-1, 3)]) * coeff
    n = len(x)
    na = len(a)
    mass = np.r_[np.full(na, params[0][0]), np.full(n - na, params[1][0])]
    mu = np.r_[np.full(na, 3e3 / (2 * 1.3)), np.full(n - na, 6e3 / (2 * 1.25))]
    lam = np.r_[np.full(na, 3e3 * 0.3 / (1.3 * 0.4)), np.full(n - na, 6e3 * 0.25 / (1.25 * 0.5))]
    v = np.zeros((n, 3)); F = np.tile(np.eye(3), (n, 1, 1)); C = np.zeros((n, 3, 3)); Jp = np.ones((n, 1))
    worst = 0.0
    for k in range(1, steps + 1):
        O.substep_3d(32, 32.0, 1.0, 1 / 32, 1e-4, 1e-5, -9.8, x, mass, mu, lam, v, F, C, Jp)
        got = sim.displacements[k].reshape(-1, 3) * coeff
        worst = max(worst, float(np.abs(got - x).max()))
    assert worst < 5e-6, worst
    np.testing.assert_allclose(np.load(tmp_path / "out" / f"{steps}.npy"), sim.displacements[-1])


def test_simulation_without_displacements_matches_the_run_with_them():
    coeff = 0.5
    a = generate_cube_points((0.5, 0.9), (0.6, 1.0), (0.5, 0.9), 10)
    runs = []
    for save in (True, False):
        sim = MPMSimulation("", 90, 1e-4, 2e-5, 1e-5, 1e-5, -9.8, 3e3, 6e3, 0.3, 0.25, 1.0, 32, coeff,
                            save_displacements=save, chunk=40)
        sim.load(meshes=[_Mesh(a)], params=[(2e-5, 3e3, 0.3)])
        sim.run()
        runs.append(sim.solver.positions().double().cpu().numpy())
    assert np.abs(runs[0] - runs[1]).max() < 1e-6


def test_load_rejects_length_mismatch():
    sim = MPMSimulation("", 1, 1e-4, 1, 1, 1, -9.8, 1e3, 1e3, 0.3, 0.3, 1.0, 16, 1.0)
    with pytest.raises(ValueError):
        sim.load(meshes=[_Mesh(np.zeros((1, 3)) + 0.5)], params=[])
