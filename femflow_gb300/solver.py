"""Resident MLS-MPM solver: the state lives in HBM, physically sorted by grid block.

``MPMSolver`` is the fast path behind ``MPMSimulation`` (femflow/simulation/mpm/simulation.py:
122-149 steps ``solve_mls_mpm_3d`` in a loop).  Each substep is the same arithmetic as
``solve_mls_mpm_3d``; the difference is that G2P writes the particles back in block-sorted
order (ping-pong buffers ``a``/``b``), so the next substep's gathers are coalesced, and that many
substeps run per host call (optionally replayed from a CUDA graph).  Particle ids travel with
the state, so ``state()`` returns arrays in the caller's original order.
"""
from __future__ import annotations

import ctypes

import torch

from . import _native as N
from . import engine as E


class _Buffers:
    """One particle state, component-major: x/v are [dim, n], F/C are [dim*dim, n] (row-major
    matrix entries), so that every per-component access of a warp is coalesced."""

    def __init__(self, n, dim, dtype, device, per_particle_material):
        z = lambda *s: torch.empty(s, dtype=dtype, device=device)
        self.n, self.dim = n, dim
        self.x, self.v = z(dim, n), z(dim, n)
        self.F, self.C = z(dim * dim, n), z(dim * dim, n)
        self.Jp = z(n)
        if per_particle_material:
            self.mass, self.mu_0, self.lambda_0 = z(n), z(n), z(n)
        else:
            self.mass = self.mu_0 = self.lambda_0 = None
        self.ids = torch.empty(n, dtype=torch.int32, device=device)

    def struct(self) -> N.Particles:
        return E.particles_struct(self.x, self.v, self.F, self.C, self.Jp, self.mass, self.mu_0, self.lambda_0,
                                  stride=self.n, n=self.n)

    def rows(self):
        """The state as row-major (reference-layout) tensors, in buffer order."""
        n, d = self.n, self.dim
        return dict(x=self.x.T.contiguous(), v=self.v.T.contiguous(), F=self.F.T.reshape(n, d, d).contiguous(),
                    C=self.C.T.reshape(n, d, d).contiguous(), Jp=self.Jp.clone())


class MPMSolver:
    """Block-sorted resident state + substep driver.

    Args mirror ``solve_mls_mpm_3d`` (mls_mpm.py:40-53) plus the 2D scalars of two_d.p2g:
    ``dim``, ``res``, ``dt``, ``gravity``, ``volume``, ``hardening``; material either per particle
    (``mass``, ``mu_0``, ``lambda_0`` tensors) or scalar.  ``sort_every``: substeps between re-sorts
    by block (with separate G2P and P2G launches a particle that leaves the blocks around its own
    triggers an earlier one; the fused path handles such particles in place; the deterministic mode
    re-sorts every substep).  Every ``step`` call (and every replay of a captured graph) starts with
    a sort, so calls whose length is a multiple of ``sort_every`` re-sort exactly every
    ``sort_every`` substeps.  ``planes``: up to 8 planar colliders (point, normal) that every grid
    update applies (three_d/grid_op.py:50-67; ``plane_rule`` "sticky" or "reference_literal").
    """

    def __init__(self, x, *, res: int, dt: float, gravity: float = -9.8, volume: float = 1.0,
                 hardening: float = 1.0, mass=1.0, mu_0=0.0, lambda_0=0.0, v=None, F=None, C=None, Jp=None,
                 dtype=torch.float32, device="cuda", model="neo_hookean", wall_mode="reference",
                 block_size: int = 0, variant: int = 0, deterministic: bool = False, sort_every: int = 8,
                 planes=None, plane_rule: str = "sticky"):
        E._require_cuda()
        device = torch.device(device)
        x = torch.as_tensor(x)
        n, dim = int(x.shape[0]), int(x.shape[1])
        per_particle = isinstance(mass, torch.Tensor) or hasattr(mass, "__len__")
        self.n, self.dim, self.dtype, self.device = n, dim, dtype, device
        dx = 1.0 / res
        self.params = E.make_params(dim, res, dtype, dx, float(res), dt, gravity, volume, hardening,
                                    0.0 if per_particle else float(mass), 0.0 if per_particle else float(mu_0),
                                    0.0 if per_particle else float(lambda_0), model=model, wall_mode=wall_mode,
                                    block_size=block_size,
                                    variant=(variant & 0xFF) | (max(1, min(255, int(sort_every))) << 8),
                                    deterministic=deterministic, planes=planes, plane_rule=plane_rule)
        self._a = _Buffers(n, dim, dtype, device, per_particle)
        self._b = _Buffers(n, dim, dtype, device, per_particle)
        a = self._a
        a.x.copy_(x.to(device=device, dtype=dtype).T)
        a.v.copy_((torch.zeros(n, dim) if v is None else torch.as_tensor(v).reshape(n, dim)).T)
        Fr = torch.eye(dim).expand(n, dim, dim) if F is None else torch.as_tensor(F).reshape(n, dim, dim)
        a.F.copy_(Fr.reshape(n, dim * dim).T)
        Cr = torch.zeros(n, dim, dim) if C is None else torch.as_tensor(C).reshape(n, dim, dim)
        a.C.copy_(Cr.reshape(n, dim * dim).T)
        a.Jp.copy_(torch.ones(n) if Jp is None else torch.as_tensor(Jp).reshape(n))
        if per_particle:
            a.mass.copy_(torch.as_tensor(mass).reshape(n))
            a.mu_0.copy_(torch.as_tensor(mu_0).reshape(n))
            a.lambda_0.copy_(torch.as_tensor(lambda_0).reshape(n))
        a.ids.copy_(torch.arange(n, dtype=torch.int32))
        self.ws = E.Workspace(self.params, n, device)
        self._cur, self._oth = self._a, self._b
        self.steps_done = 0
        self._graph = None
        self._graph_steps = 0

    # ------------------------------------------------------------------ stepping
    def _call(self, nsteps: int, stream_ptr: int, snapshots=None):
        sa, sb = self._cur.struct(), self._oth.struct()
        head = (ctypes.byref(self.params), ctypes.byref(sa), ctypes.byref(sb),
                ctypes.c_void_p(self._cur.ids.data_ptr()), ctypes.c_void_p(self._oth.ids.data_ptr()), int(nsteps))
        tail = (ctypes.c_void_p(self.ws.ptr), ctypes.c_size_t(self.ws.bytes), ctypes.c_void_p(stream_ptr))
        if snapshots is None:
            N.call("ffmpm_substeps_sorted", *head, *tail)
        else:
            sx, si = snapshots
            if sx.shape[0] < nsteps or si.shape[0] < nsteps or sx.dtype != self.dtype or si.dtype != torch.int32:
                raise ValueError("snapshot arrays: x [>= nsteps, dim, n] of the solver's dtype, ids [>= nsteps, n] int32")
            N.call("ffmpm_substeps_sorted_snapshots", *head, ctypes.c_void_p(sx.data_ptr()),
                   ctypes.c_void_p(si.data_ptr()), *tail)

    def _launch(self, nsteps: int, snapshots=None):
        self._call(nsteps, E._stream_ptr(self.device), snapshots)
        if nsteps % 2 == 1:
            self._cur, self._oth = self._oth, self._cur
        self.steps_done += nsteps

    def step(self, nsteps: int = 1, check: bool = False, snapshots=None):
        """Run ``nsteps`` substeps (stream-ordered, asynchronous unless ``check``).  ``snapshots``:
        device arrays (x [>= nsteps, dim, n] of the solver's dtype, ids [>= nsteps, n] int32) that
        receive every substep's positions in block-sorted order and the ids that go with them (the
        positions of particle ids[k][i] are x[k][:, i]); a captured graph replays with the arrays
        it was captured with."""
        if self._graph is not None and nsteps % self._graph_steps == 0 and snapshots is None:
            for _ in range(nsteps // self._graph_steps):
                self._graph.replay()
            self.steps_done += nsteps
        else:
            self._launch(nsteps, snapshots)
        if check:
            self.ws.raise_on_status()

    def capture(self, nsteps: int, snapshots=None, warmup: bool = True):
        """Capture ``nsteps`` (even) substeps into a CUDA graph; ``step`` then replays it (with the
        ``snapshots`` arrays, when given).  ``warmup`` first runs two substeps directly, so that the
        first-call set-up happens outside the capture; pass False when the solver has run before."""
        if nsteps <= 0 or nsteps % 2:
            raise ValueError("graph capture needs an even number of substeps (state returns to its buffer)")
        if warmup:
            self._launch(2)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self._call(nsteps, s.cuda_stream, snapshots)
        torch.cuda.synchronize(self.device)
        self._graph, self._graph_steps = g, nsteps
        return g

    def profile(self, nsteps: int) -> dict:
        """Run ``nsteps`` substeps with CUDA events around every phase (synchronises).

        Returns {phase: (total_ms, launches)} for keys, sort, plan, p2g, grid_update, g2p and g2p2g
        (the fused G2P + next substep's P2G).
        """
        ms = (ctypes.c_double * N.NPHASES)()
        cnt = (ctypes.c_int64 * N.NPHASES)()
        sa, sb = self._cur.struct(), self._oth.struct()
        N.call("ffmpm_profile_substeps", ctypes.byref(self.params), ctypes.byref(sa), ctypes.byref(sb),
               ctypes.c_void_p(self._cur.ids.data_ptr()), ctypes.c_void_p(self._oth.ids.data_ptr()), int(nsteps),
               ctypes.c_void_p(self.ws.ptr), ctypes.c_size_t(self.ws.bytes),
               ctypes.c_void_p(E._stream_ptr(self.device)), ms, cnt)
        if nsteps % 2 == 1:
            self._cur, self._oth = self._oth, self._cur
        self.steps_done += nsteps
        return {N.PHASES[i]: (ms[i], cnt[i]) for i in range(N.NPHASES)}

    def plan_info(self) -> dict:
        info = (ctypes.c_int64 * 8)()
        N.call("ffmpm_plan_info", ctypes.byref(self.params), self.n, info)
        keys = ("block_size", "blocks_per_axis", "blocks", "key_bits", "radix_passes", "kernels_per_substep",
                "tile", "max_chunks")
        return dict(zip(keys, list(info)))

    def kernels_per_call(self, nsteps: int) -> int:
        """Kernels one call of ``nsteps`` substeps launches (as counted by the library)."""
        c = ctypes.c_int64()
        N.call("ffmpm_kernels_per_call", ctypes.byref(self.params), self.n, int(nsteps), ctypes.byref(c))
        return int(c.value)

    # ------------------------------------------------------------------ state access
    def sorted_state(self):
        """State in the current (block-sorted) buffer order, as row-major copies, with the ids."""
        c = self._cur
        out = c.rows()
        out.update(ids=c.ids, mass=c.mass, mu_0=c.mu_0, lambda_0=c.lambda_0)
        return out

    def state(self):
        """State in the original particle order, row-major (new tensors)."""
        c = self._cur
        ids = c.ids.long()
        out = {}
        for k, t in c.rows().items():
            o = torch.empty_like(t)
            o[ids] = t
            out[k] = o
        return out

    def positions(self):
        return self.state()["x"]

    def status(self):
        return self.ws.status()

    def check(self):
        self.ws.raise_on_status()

    def diagnostics(self) -> dict:
        """Float64 energies / momentum / mass / min det F of the current state."""
        out = torch.zeros(8, dtype=torch.float64, device=self.device)
        s = self._cur.struct()
        N.call("ffmpm_diagnostics_fp64", ctypes.byref(self.params), ctypes.byref(s), ctypes.c_void_p(out.data_ptr()),
               ctypes.c_void_p(E._stream_ptr(self.device)))
        o = out.cpu().tolist()
        return dict(kinetic=o[0], elastic=o[1], gravitational=o[2], momentum=o[3:6], mass=o[6], min_det_F=o[7])
