"""GPU-resident ``MPMSimulation`` (femflow/simulation/mpm/simulation.py:19-149).

Same constructor, ``load(meshes=, params=)``, ``start()``, ``reset()``, ``displacements`` and
per-step ``.npy`` output as the reference.  The particle state stays on the GPU in the
block-sorted resident solver (``MPMSolver``), stepped in chunks of ``chunk`` substeps (a multiple
of its re-sort cadence) replayed from a captured CUDA graph.  The solver keeps every substep's
positions in device snapshot arrays; each is put back into the caller's particle order on the GPU
(and into the reference's float64 / tightening_coeff form), sent to one of a few reused pinned
host buffers on a copy stream, and appended to ``displacements`` as soon as its copy has
completed, so that a reader (the reference's GUI thread, gui.py:38-39) sees the run's progress
while it goes on, as with simulation.py:140-142.  As in the reference, the constructor's ``force``
is what the substep receives as gravity (simulation.py:126-139) and the constructor's ``volume``
is the particle volume.
"""
from __future__ import annotations

import collections
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
                 dtype=torch.float32, device="cuda", chunk: int = 40, host_buffers: int = 8):
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
        self.chunk, self.host_buffers = int(chunk), int(host_buffers)
        if self.chunk < 2 or self.chunk % 2 or self.host_buffers < 1:
            raise ValueError("chunk must be even and at least 2, host_buffers at least 1")
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
        if self.save_displacements:
            self._run_with_snapshots(steps)
        else:
            self._run(steps)
        self.solver.check()
        if self.save_displacements and self.outdir:
            log.info("Saving displacements")
            os.makedirs(self.outdir, exist_ok=True)
            for i, d in enumerate(self.displacements):
                np.save(os.path.join(self.outdir, str(i)), d)
        log.info("Simulation done")
        self.running = False

    def _run(self, steps: int):
        """Chunks of ``chunk`` substeps from a captured graph, the remainder directly."""
        solver, K = self.solver, self.chunk
        done = 0
        if steps >= 2 * K:
            solver.step(K)  # first-call set-up outside the capture
            solver.capture(K, warmup=False)
            done = K
        while steps - done >= K:
            solver.step(K)
            done += K
        if steps > done:
            solver.step(steps - done)

    def _run_with_snapshots(self, steps: int):
        solver, K, coeff = self.solver, min(self.chunk, max(steps, 1)), self.tightening_coeff
        dev = torch.device(self.device)
        n, dim = solver.n, solver.dim
        snap = (torch.empty((K, dim, n), dtype=self.dtype, device=dev), torch.empty((K, n), dtype=torch.int32, device=dev))
        R = self.host_buffers
        dev_ring = [torch.empty((n, dim), dtype=torch.float64, device=dev) for _ in range(R)]
        host_ring = [torch.empty((n, dim), dtype=torch.float64, pin_memory=True) for _ in range(R)]
        free = collections.deque(range(R))
        pending = collections.deque()  # (copy-completed event, ring slot), in substep order
        compute = torch.cuda.current_stream(dev)
        copy_stream = torch.cuda.Stream(dev)

        def drain(wait_for_one: bool):
            while pending and (wait_for_one or pending[0][0].query()):
                ev, slot = pending.popleft()
                ev.synchronize()
                self.displacements.append(host_ring[slot].numpy().reshape(-1).copy())
                free.append(slot)
                wait_for_one = False

        done, captured = 0, False
        while done < steps:
            k_n = min(K, steps - done)
            if captured and k_n == K:
                solver.step(K)
            else:
                solver.step(k_n, snapshots=snap)
                if not captured and k_n == K and steps - done - K >= K:
                    solver.capture(K, snapshots=snap, warmup=False)
                    captured = True
            for k in range(k_n):
                if not free:
                    drain(True)
                slot = free.popleft()
                # the caller's order (row ids[i] <- column i) and the reference's form, on the GPU
                dev_ring[slot].index_copy_(0, snap[1][k].long(), snap[0][k].t().double())
                dev_ring[slot].div_(coeff)
                ready = torch.cuda.Event()
                ready.record(compute)
                with torch.cuda.stream(copy_stream):
                    copy_stream.wait_event(ready)
                    host_ring[slot].copy_(dev_ring[slot], non_blocking=True)
                    copied = torch.cuda.Event()
                    copied.record(copy_stream)
                pending.append((copied, slot))
                drain(False)
            done += k_n
        while pending:
            drain(True)
