"""Batched 2D scenes: many independent MLS-MPM scenes advanced by one persistent launch per call.

Each scene has its own particles, grid resolution, material (two_d.p2g's scalar ``mass``,
``mu_0``, ``lambda_0``), dt, gravity and walls.  The particle state of all scenes lives in one set
of component-major arrays, each scene's particles ordered by base cell (``scene_state`` returns
them in the caller's order).  ``step`` runs any number of substeps in one cooperative launch (P2G,
then per substep the grid update over each scene's box of touched nodes and G2P fused with the
next P2G, grid-wide barriers in between), ``capture`` records such a launch in a CUDA graph, and
``autotune`` picks the launch shape.
"""
from __future__ import annotations

import ctypes
from typing import Dict, List

import numpy as np
import torch

from . import _native as N
from . import autotune as AT
from . import engine as E


class Scene2D(ctypes.Structure):
    _fields_ = [("offset", ctypes.c_int64), ("count", ctypes.c_int64), ("res", ctypes.c_int32),
                ("model", ctypes.c_int32), ("wall_mode", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("dx", ctypes.c_double), ("inv_dx", ctypes.c_double), ("dt", ctypes.c_double),
                ("gravity", ctypes.c_double), ("volume", ctypes.c_double), ("hardening", ctypes.c_double),
                ("mass", ctypes.c_double), ("mu_0", ctypes.c_double), ("lambda_0", ctypes.c_double)]


def batch_cell_order(x: np.ndarray, offsets, res) -> np.ndarray:
    """perm[i] = the caller's index (within the batch) of the particle at position i: every scene's
    particles (x[offsets[s]:offsets[s+1]] on a res[s]^2 grid) stably ordered by base cell, scenes
    kept in place."""
    perm = []
    for s, r in enumerate(res):
        a, b = int(offsets[s]), int(offsets[s + 1])
        cell = np.clip(np.floor(x[a:b] * r - 0.5), -1, r).astype(np.int64)
        perm.append(a + np.argsort(cell[:, 0] * (r + 2) + cell[:, 1], kind="stable"))
    return np.concatenate(perm) if perm else np.zeros(0, dtype=np.int64)


class Batch2D:
    """``scenes``: list of dicts with ``x`` [n,2] and scalars ``res``, ``dt``, ``mass``, ``volume``,
    ``mu_0``, ``lambda_0`` (optional: ``v``, ``F``, ``C``, ``Jp``, ``gravity`` (-9.8),
    ``hardening`` (1), ``model`` ("neo_hookean"), ``wall_mode`` ("reference"))."""

    def __init__(self, scenes: List[Dict], dtype=torch.float32, device="cuda"):
        E._require_cuda()
        if not 1 <= len(scenes) <= 256:
            raise ValueError("a batch holds 1..256 scenes")
        self.dtype, self.device = dtype, torch.device(device)
        self.nscenes = len(scenes)
        counts = [int(np.asarray(s["x"]).shape[0]) for s in scenes]
        self.offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        n = int(self.offsets[-1])
        self.n = n
        cat = lambda key, shape, default: np.concatenate([
            np.asarray(s[key], dtype=np.float64).reshape(-1, *shape) if key in s and s[key] is not None else
            default(c) for s, c in zip(scenes, counts)])
        x = cat("x", (2,), lambda c: np.zeros((c, 2)))
        v = cat("v", (2,), lambda c: np.zeros((c, 2)))
        F = cat("F", (2, 2), lambda c: np.tile(np.eye(2), (c, 1, 1)))
        C = cat("C", (2, 2), lambda c: np.zeros((c, 2, 2)))
        Jp = np.concatenate([np.asarray(s.get("Jp", np.ones(c)), dtype=np.float64).reshape(-1)
                             for s, c in zip(scenes, counts)])
        # each scene's particles in the order of their base cell: the kernel's P2G sums the
        # contributions of a warp's lanes that share a cell before its atomics
        perm = batch_cell_order(x, self.offsets, [int(s["res"]) for s in scenes])
        x, v, F, C, Jp = x[perm], v[perm], F[perm], C[perm], Jp[perm]
        self.perm = torch.as_tensor(perm, device=self.device)
        self._inv = torch.empty_like(self.perm)
        self._inv[self.perm] = torch.arange(n, device=self.device)
        dev = lambda a: torch.tensor(a, dtype=dtype, device=self.device)
        self.x, self.v = dev(x.T.copy()), dev(v.T.copy())
        self.F, self.C = dev(F.reshape(n, 4).T.copy()), dev(C.reshape(n, 4).T.copy())
        self.Jp = dev(Jp)
        table = (Scene2D * self.nscenes)()
        for i, s in enumerate(scenes):
            t = table[i]
            t.offset, t.count = int(self.offsets[i]), counts[i]
            t.res = int(s["res"])
            t.model = N.MODELS[s.get("model", "neo_hookean")]
            t.wall_mode = N.WALLS[s.get("wall_mode", "reference")]
            t.dx, t.inv_dx = 1.0 / t.res, float(t.res)
            t.dt, t.gravity = float(s["dt"]), float(s.get("gravity", -9.8))
            t.volume, t.hardening = float(s["volume"]), float(s.get("hardening", 1.0))
            t.mass, t.mu_0, t.lambda_0 = float(s["mass"]), float(s["mu_0"]), float(s["lambda_0"])
        self.table = table
        self.rb = E.real_bytes(dtype)
        nbytes = ctypes.c_size_t(0)
        tptr = ctypes.c_void_p(ctypes.addressof(table))
        N.call("ffmpm_batch2d_workspace_size", tptr, self.nscenes, self.rb, ctypes.byref(nbytes))
        self.ws_bytes = int(nbytes.value)
        self._wsbuf = torch.empty(self.ws_bytes + 256, dtype=torch.uint8, device=self.device)
        self.ws = (self._wsbuf.data_ptr() + 255) // 256 * 256
        N.call("ffmpm_batch2d_init", tptr, self.nscenes, self.rb, ctypes.c_void_p(self.ws),
               ctypes.c_size_t(self.ws_bytes), ctypes.c_void_p(E._stream_ptr(self.device)))
        self.threads, self.ctas_per_sm = 256, 0
        self._graph, self._graph_steps = None, 0

    def _struct(self):
        return E.particles_struct(self.x, self.v, self.F, self.C, self.Jp, stride=self.n, n=self.n)

    def _launch(self, nsteps: int, threads=None, ctas=None, stream=None):
        st = self._struct()
        N.call("ffmpm_batch2d_substeps", self.nscenes, self.rb, ctypes.byref(st), int(nsteps),
               int(threads or self.threads), int(self.ctas_per_sm if ctas is None else ctas),
               ctypes.c_void_p(self.ws), ctypes.c_size_t(self.ws_bytes),
               ctypes.c_void_p(stream if stream is not None else E._stream_ptr(self.device)))

    def step(self, nsteps: int = 1):
        if self._graph is not None and nsteps % self._graph_steps == 0:
            for _ in range(nsteps // self._graph_steps):
                self._graph.replay()
        else:
            self._launch(nsteps)

    def capture(self, nsteps: int):
        """Record `nsteps` substeps (one cooperative launch) in a CUDA graph."""
        self._launch(1)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self._launch(nsteps, stream=s.cuda_stream)
        torch.cuda.synchronize(self.device)
        self._graph, self._graph_steps = g, nsteps
        return g

    def autotune(self, steps: int = 2):
        """Choose (threads per CTA, CTAs per SM) by timing `steps` substeps of this batch per
        candidate.  The state advances by the substeps used for timing."""
        sig = ("batch2d", self.nscenes, self.n, int(sum((t.res + 1) ** 2 for t in self.table)), self.rb)
        cands = [(128, 0), (256, 0), (512, 0), (256, 2), (512, 1)]
        best, timings = AT.tune(sig, cands, lambda c: self._launch(steps, threads=c[0], ctas=c[1]))
        self.threads, self.ctas_per_sm = best
        return best, timings

    def reset(self):
        """Zero the status word, the barrier state and both grids (the scene table is kept).  A
        batch whose status shows FFMPM_STATUS_TIMEOUT holds a partly accumulated grid: reset it
        before stepping again."""
        N.call("ffmpm_batch2d_init", ctypes.c_void_p(ctypes.addressof(self.table)), self.nscenes, self.rb,
               ctypes.c_void_p(self.ws), ctypes.c_size_t(self.ws_bytes),
               ctypes.c_void_p(E._stream_ptr(self.device)))

    def set_waits(self, wait_limit: int = 0, inject: int = 0):
        """Bound of the grid-barrier waits (0: the library default) and N.INJECT_* bits, for tests
        of the bounded waits; ``reset`` restores both to 0."""
        N.call("ffmpm_batch2d_set_waits", ctypes.c_void_p(self.ws), int(wait_limit), int(inject),
               ctypes.c_void_p(E._stream_ptr(self.device)))

    def status(self) -> int:
        st = ctypes.c_int32(0)
        N.call("ffmpm_batch2d_status", ctypes.c_void_p(self.ws), ctypes.byref(st),
               ctypes.c_void_p(E._stream_ptr(self.device)))
        return int(st.value)

    def scene_state(self, i: int) -> Dict[str, torch.Tensor]:
        """Scene i's state in the caller's particle order (the batch keeps it ordered by cell)."""
        a, b = int(self.offsets[i]), int(self.offsets[i + 1])
        c = b - a
        pos = self._inv[a:b]  # where the scene's particles sit in the batch, in the caller's order
        return dict(x=self.x[:, pos].T.contiguous(), v=self.v[:, pos].T.contiguous(),
                    F=self.F[:, pos].T.reshape(c, 2, 2).contiguous(),
                    C=self.C[:, pos].T.reshape(c, 2, 2).contiguous(), Jp=self.Jp[pos].clone())

    def position(self, i: int, k: int) -> int:
        """Index in the batch arrays of the caller's particle k of scene i."""
        return int(self._inv[int(self.offsets[i]) + k])


def random_scenes(nscenes: int = 256, seed: int = 0, n_range=(2048, 65536), res_range=(64, 256),
                  E_range=(1e3, 1e5), nu_range=(0.1, 0.4), dt: float = 1e-4, edge: float = 0.2) -> List[Dict]:
    """Seeded scenes of the batched workload: particle count log-uniform in n_range, grid uniform in
    res_range, E log-uniform in E_range, nu uniform in nu_range, a square block of particles at a
    seeded position inside the domain margin, at rest."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nscenes):
        n = int(round(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1])))))
        res = int(rng.integers(res_range[0], res_range[1] + 1))
        E = float(np.exp(rng.uniform(np.log(E_range[0]), np.log(E_range[1]))))
        nu = float(rng.uniform(*nu_range))
        lo = rng.uniform(0.1, 0.9 - edge, size=2)
        x = lo + rng.uniform(0, edge, size=(n, 2))
        vol = edge * edge / n
        mu, lam = E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))
        out.append(dict(x=x, res=res, dt=dt, mass=vol, volume=vol, mu_0=mu, lambda_0=lam, E=E, nu=nu))
    return out


def stable_variant(scenes: List[Dict], cfl: float = 0.5) -> List[Dict]:
    """The same scenes with E capped so that the elastic wave crosses at most `cfl` cells per
    substep (c = sqrt((lam + 2 mu) / rho), rho = mass / volume)."""
    out = []
    for s in scenes:
        s = dict(s)
        E, nu = s["E"], s["nu"]
        rho = s["mass"] / s["volume"]
        k = (1 - nu) / ((1 + nu) * (1 - 2 * nu))  # (lam + 2 mu) / E
        E_max = rho * (cfl / (s["dt"] * s["res"])) ** 2 / k
        if E > E_max:
            E = E_max
            s["E"] = E
            s["mu_0"], s["lambda_0"] = E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))
        out.append(s)
    return out


def measure(scenes: List[Dict], steps: int = 100, reps: int = 3, sequential: bool = True) -> dict:
    """Particle-substeps/s of the batch (autotuned launch shape, `steps`-substep CUDA graph) and,
    for comparison, of the same scenes stepped one at a time on the resident single-scene solver."""
    from .solver import MPMSolver

    b = Batch2D(scenes)
    best, timings = b.autotune()
    b.capture(steps)
    b.step(steps)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    b.step(steps * reps)
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    out = dict(scenes=len(scenes), particles=b.n, substeps=steps * reps, graph_substeps=steps,
               launch_shape=dict(threads=best[0], ctas_per_sm=best[1]),
               autotune_ms={f"{k[0]}x{k[1]}": v for k, v in timings.items()},
               batched=dict(seconds=t, particle_substeps_per_s=b.n * steps * reps / t), status=b.status())
    if sequential:
        solvers = [MPMSolver(torch.tensor(s["x"]), res=s["res"], dt=s["dt"], gravity=-9.8, volume=s["volume"],
                             mass=s["mass"], mu_0=s["mu_0"], lambda_0=s["lambda_0"], dtype=torch.float32)
                   for s in scenes]
        for sv in solvers:
            sv.step(2)
        torch.cuda.synchronize()
        e0.record()
        for sv in solvers:
            sv.step(steps)
        e1.record()
        torch.cuda.synchronize()
        ts = e0.elapsed_time(e1) / 1e3
        out["one_scene_at_a_time"] = dict(seconds=ts, particle_substeps_per_s=b.n * steps / ts)
        out["speedup_batched"] = out["batched"]["particle_substeps_per_s"] / out["one_scene_at_a_time"][
            "particle_substeps_per_s"]
    return out


def main(argv=None):
    import argparse
    import json

    ap = argparse.ArgumentParser(description="throughput of the batched 2D scenes")
    ap.add_argument("--scenes", type=int, default=256)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--profile-case", action="store_true",
                    help="stable variant, 256 threads per CTA: one launch of 3 substeps, then one launch of "
                         "--steps substeps (the one to capture with a profiler); prints the status")
    a = ap.parse_args(argv)
    sc = random_scenes(a.scenes, seed=a.seed)
    if a.profile_case:
        b = Batch2D(stable_variant(sc), dtype=torch.float32)
        b.threads, b.ctas_per_sm = 256, 0
        b.step(3)
        torch.cuda.synchronize()
        b.step(a.steps)
        torch.cuda.synchronize()
        print(json.dumps({"particles": b.n, "substeps": a.steps, "status": b.status()}))
        return
    rep = {"as_written": measure(sc, a.steps, sequential=False), "stable_variant": measure(stable_variant(sc), a.steps)}
    print(json.dumps(rep, indent=1, default=float))


if __name__ == "__main__":
    main()
