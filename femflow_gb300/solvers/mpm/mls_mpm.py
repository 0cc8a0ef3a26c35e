"""Mirror of ``femflow.solvers.mpm.mls_mpm`` (femflow/solvers/mpm/mls_mpm.py)."""
from __future__ import annotations

import ctypes

import torch

from ... import engine as E
from . import _phase as P


def make_mls_mpm_coefficients(lenx: int, dim: int, dtype=torch.float32, device="cuda"):
    """mls_mpm.py:9-15: v = 0 [N,dim], F = I [N,dim,dim], C = 0 [N,dim,dim], Jp = 1 [N,1].

    The reference returns float64 numpy arrays; here the arrays are tensors on ``device``
    (float32 on the GPU by default; pass ``dtype=torch.float64`` for the float64 path).
    """
    v = torch.zeros((lenx, dim), dtype=dtype, device=device)
    F = torch.eye(dim, dtype=dtype, device=device).repeat(lenx, 1, 1).contiguous()
    C = torch.zeros((lenx, dim, dim), dtype=dtype, device=device)
    Jp = torch.ones((lenx, 1), dtype=dtype, device=device)
    return v, F, C, Jp


def solve_mls_mpm_3d(res, inv_dx, hardening, dx, dt, volume, gravity, particles, v, F, C, Jp, *,
                     check: bool = True, deterministic: bool = False):
    """mls_mpm.py:40-79: one substep (p2g, grid_op, g2p on a fresh (res+1)^3 grid), in place.

    ``particles`` is a ``ParticleSet`` (or a list of ``Particle``, converted on the host).  The
    model is fixed to "neo_hookean" as in mls_mpm.py:58.  Host arrays are staged to the GPU and
    written back; pinned CPU tensors of one dtype take ffmpm_substep_host, whose copies run while
    its kernels do.  Raises RuntimeError when a particle leaves the grid.
    """
    pset, plist = P.split_particles(particles)
    dtype = P.dtype_of(v, F)
    host = [pset.pos, pset.mass, pset.mu_0, pset.lambda_0, v, F, C, Jp]
    if plist is None and P.pinned_host(*host):
        E._require_cuda()
        prm = E.make_params(3, res, host[0].dtype, dx, inv_dx, dt, gravity, volume, hardening, model="neo_hookean",
                            deterministic=deterministic)
        P.run_host_substep(prm, *host, check=check)
        return
    st = E.stage([pset.pos, pset.mass, pset.mu_0, pset.lambda_0, v, F, C, Jp], dtype=dtype)
    x, m, mu, lam, vv, FF, CC, JJ = st.dev
    E.check_tensors(dtype, x, m, mu, lam, vv, FF, CC, JJ)
    prm = E.make_params(3, res, dtype, dx, inv_dx, dt, gravity, volume, hardening, model="neo_hookean",
                        deterministic=deterministic)
    ps = E.particles_struct(x, vv, FF, CC, JJ, m, mu, lam)
    P.run("ffmpm_substep", prm, ps.n, x.device, ctypes.byref(prm), ctypes.byref(ps), check=check)
    st.write_back([0, 4, 5, 6, 7])
    if plist is not None:
        pset.write_positions(plist)
