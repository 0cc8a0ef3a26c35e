"""GPU-resident ``MPMSimulation`` (femflow/simulation/mpm/simulation.py:19-149).

Same constructor, ``load(meshes=, params=)``, ``start()``, ``reset()``, ``displacements`` and
per-step ``.npy`` output as the reference.  The particle state stays on the GPU in the
block-sorted resident solver (``MPMSolver``); positions are copied to pinned host buffers
asynchronously after every substep, in the caller's particle order.  As in the reference, the
constructor's ``force`` is what the substep receives as gravity (simulation.py:126-139) and the
constructor's ``volume`` is the particle volume.
"""
from __future__ import annotations

import logging
import os
import threading
from typing import List, Sequence, Tuple

import numpy as np
import torch

from ...solver import MPMSolver
from ...solvers.mpm.utils import Ev_to_lambda, Ev_to_mu

log = logging.getLogger("femflow_gb300")


def _vertices(mesh) -> np.ndarray:
    v = mesh.vertices if hasattr(mesh, "vertices") else mesh
    return np.asarray(v, dtype=np.float64).reshape(-1, 3)


class MPMSimulation:
    def __init__(self, outdir: str, steps: int, dt: float, gyroid_mass: float, collider_mass: float, volume: float,
                 force: float, gyroid_E: float, collider_E: float, gyroid_v: float, collider_v: float,
                 hardening: float, grid_res: int, tightening_coeff: float, save_displacements: bool = True,
                 dtype=torch.float32, device="cuda"):
        self.outdir = outdir
        self.save_displacements = save_displacements
        self.loaded = False
        self.running = False
        self.displacements: List[np.ndarray] = []
        self.steps, self.dt = steps, dt
        self.gyroid_mass, self.collider_mass, self.volume, self.force = gyroid_mass, collider_mass, volume, force
        self.gyroid_E, self.collider_E, self.gyroid_v, self.collider_v = gyroid_E, collider_E, gyroid_v, collider_v
        self.hardening, self.grid_res, self.tightening_coeff = hardening, grid_res, tightening_coeff
        self.gyroid_mu_0 = self.gyroid_E / (2 * (1 + self.gyroid_v))
        self.gyroid_lambda_0 = self.gyroid_E * self.gyroid_v / ((1 + self.gyroid_v) * (1 - 2 * self.gyroid_v))
        self.dx = 1 / self.grid_res
        self.inv_dx = 1 / self.dx
        self.dtype, self.device = dtype, device
        self.solver: MPMSolver | None = None
        self._thread: threading.Thread | None = None

    def load(self, **kwargs):
        """simulation.py:68-111: particles = mesh vertices x tightening_coeff, material per mesh."""
        meshes: Sequence = kwargs["meshes"]
        params: Sequence[Tuple[float, float, float]] = kwargs["params"]
        if len(meshes) != len(params):
            raise ValueError(f"Meshes {len(meshes)} and Params  {len(params)} must be the same length")
        xs, mass, mu, lam = [], [], [], []
        for mesh, (m, E, nu) in zip(meshes, params):
            v = _vertices(mesh) * self.tightening_coeff
            xs.append(v)
            mass.append(np.full(len(v), m))
            lam.append(np.full(len(v), Ev_to_lambda(E, nu)))
            mu.append(np.full(len(v), Ev_to_mu(E, nu)))
        x = np.concatenate(xs)
        self.n = len(x)
        self.solver = MPMSolver(torch.tensor(x), res=self.grid_res, dt=self.dt, gravity=self.force, volume=self.volume,
                                hardening=self.hardening, mass=torch.tensor(np.concatenate(mass)),
                                mu_0=torch.tensor(np.concatenate(mu)), lambda_0=torch.tensor(np.concatenate(lam)),
                                dtype=self.dtype, device=self.device)
        self.displacements = [x.reshape(-1) / self.tightening_coeff] if self.save_displacements else []
        self.loaded = True
        log.info("Simulation loaded: %d particles", self.n)

    def start(self, **kwargs):
        if not self.loaded:
            log.error("Please load the simulation first")
            return
        self._thread = threading.Thread(target=self._simulate_offline, daemon=True)
        self._thread.start()

    def join(self, timeout: float | None = None):
        if self._thread is not None:
            self._thread.join(timeout)

    def reset(self, **kwargs):
        self.load(**kwargs)

    def run(self, steps: int | None = None):
        """The substep loop of simulation.py:122-149 on the calling thread."""
        self._simulate_offline(steps)

    def _simulate_offline(self, steps: int | None = None):
        self.running = True
        steps = self.steps if steps is None else steps
        dev = torch.device(self.device)
        copy_stream = torch.cuda.Stream(dev)
        pending = []
        for _ in range(steps):
            self.solver.step(1)
            if self.save_displacements:
                # positions in the caller's order, copied to pinned memory off the compute stream
                pos = self.solver.positions()
                host = torch.empty(pos.shape, dtype=pos.dtype, pin_memory=True)
                ev = torch.cuda.Event()
                ev.record()
                with torch.cuda.stream(copy_stream):
                    copy_stream.wait_event(ev)
                    host.copy_(pos, non_blocking=True)
                    pos.record_stream(copy_stream)
                pending.append(host)
        copy_stream.synchronize()
        self.solver.check()
        for host in pending:
            self.displacements.append(host.double().numpy().reshape(-1) / self.tightening_coeff)
        if self.save_displacements and self.outdir:
            log.info("Saving displacements")
            os.makedirs(self.outdir, exist_ok=True)
            for i, d in enumerate(self.displacements):
                np.save(os.path.join(self.outdir, str(i)), d)
        log.info("Simulation done")
        self.running = False
