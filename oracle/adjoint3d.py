"""FP64 numpy restatement of the 3D MLS-MPM substep and of its adjoint — test infrastructure only.

The forward half restates ``solve_mls_mpm_3d`` (femflow/solvers/mpm/mls_mpm.py:40-79) with the
"neo_hookean" model (fixed-corotated stress, constant hardening) vectorised over particles:

* P2G    three_d/p2g.py:14-80      base = trunc(x*inv_dx - 0.5), quadratic B-spline weights,
                                     A = -dt*vol*4*inv_dx^2*PF + m*C with
                                     PF = 2mu(F-R)F^T + lam(J-1)J on all nine entries (utils.py:95-135)
                                     or, with ``lam_diagonal``, on the diagonal only (the textbook
                                     fixed-corotated stress, model "fixed_corotated" of the C oracle),
                                     R = U Vh from the SVD of F (linear_algebra.py:119-135)
* grid   three_d/grid_op.py:5-47   v = p/m, v_y += dt*g, clip to +-0.9dx/dt, zero the normal
                                     component on the 1-cell wall band (all nodes)
* G2P    three_d/g2p.py:9-59       v, C = 4*inv_dx*sum w*v_i (x) (i - fx) (grid units),
                                     x += dt*v, F <- (I + dt*C) F

It is pinned to the C oracle (``oracle.substep_3d``), itself pinned to the reference's golden
vectors.  The reference has no derivative; the reverse half is the exact derivative of this
forward, derived by hand (reverse G2P scatters to the grid, reverse grid applies the clamp/wall
masks and the division by mass, reverse P2G gathers), including the derivative of the polar
factor: for F = R S, dL/dF gains R [y]_x with (tr(S) I - S) y = axial(R^T dL/dR).  It is pinned by
central finite differences of the forward (tests/test_adjoint_oracle.py).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

OFFS = np.array([(i, j, k) for i in range(3) for j in range(3) for k in range(3)], dtype=np.int64)  # [27,3]


@dataclass
class Params3D:
    res: int
    dt: float
    volume: float
    gravity: float = -9.8
    hardening: float = 1.0
    # False: the reference's stress, lam(J-1)J added to all nine entries of PF (utils.py:129);
    # True: the textbook fixed-corotated stress, lam(J-1)J on the diagonal only
    lam_diagonal: bool = False

    @property
    def dx(self) -> float:
        return 1.0 / self.res

    @property
    def inv_dx(self) -> float:
        return float(self.res)


def _weights(fx):
    """Quadratic B-spline weights and their derivatives in fx, each [n, 3 nodes, 3 axes]."""
    w = np.stack([0.5 * (1.5 - fx) ** 2, 0.75 - (fx - 1.0) ** 2, 0.5 * (fx - 0.5) ** 2], axis=1)
    dw = np.stack([fx - 1.5, -2.0 * (fx - 1.0), fx - 0.5], axis=1)
    return w, dw


def _stencil(x, prm):
    base = (x * prm.inv_dx - 0.5).astype(np.int64)
    if (base < 0).any() or (base + 2 > prm.res).any():
        raise RuntimeError("particle out of grid bounds")
    fx = x * prm.inv_dx - base
    w, dw = _weights(fx)
    a, b, c = OFFS[:, 0], OFFS[:, 1], OFFS[:, 2]
    W = w[:, a, 0] * w[:, b, 1] * w[:, c, 2]  # [n,27]
    dW = np.stack([dw[:, a, 0] * w[:, b, 1] * w[:, c, 2],
                   w[:, a, 0] * dw[:, b, 1] * w[:, c, 2],
                   w[:, a, 0] * w[:, b, 1] * dw[:, c, 2]], axis=2)  # [n,27,3] d/dfx
    R1 = prm.res + 1
    node = base[:, None, :] + OFFS[None]
    idx = (node[..., 0] * R1 + node[..., 1]) * R1 + node[..., 2]  # [n,27]
    rel = OFFS[None].astype(np.float64) - fx[:, None, :]  # (i - fx), grid units
    return W, dW, idx, rel


def _polar(F):
    U, s, Vh = np.linalg.svd(F)
    return U @ Vh


def _grid_masks(gv, gm, prm):
    """Grid rule of three_d/grid_op.py and the per-component pass-through mask of its derivative."""
    R1 = prm.res + 1
    n = R1 ** 3
    I = np.stack(np.unravel_index(np.arange(n), (R1, R1, R1)), axis=1)
    has = gm[:, 0] > 0
    v = gv.copy()
    v[has] /= gm[has]
    v[has, 1] += prm.dt * prm.gravity
    bound = 0.9 * prm.dx / prm.dt
    clipped = has[:, None] & ((v < -bound) | (v > bound))
    v[has] = np.clip(v[has], -bound, bound)
    wall = (I < 1) | (I >= prm.res - 1)
    v[wall] = 0.0
    keep = ~(clipped | wall)
    return v, keep, has


def forward(state, mass, mu0, lam0, prm: Params3D, tape: bool = False):
    """One substep.  state = (x[n,3], v[n,3], F[n,3,3], C[n,3,3]); mass/mu0/lam0 are [n] arrays."""
    x, v, F, C = state
    W, dW, idx, rel = _stencil(x, prm)
    dpos = rel * prm.dx
    mu = mu0 * prm.hardening
    lam = lam0 * prm.hardening
    R = _polar(F)
    J = np.linalg.det(F)
    PF = 2.0 * mu[:, None, None] * (F - R) @ np.transpose(F, (0, 2, 1)) + \
        (lam * (J - 1.0) * J)[:, None, None] * (np.eye(3)[None] if prm.lam_diagonal else 1.0)
    A = -(prm.dt * prm.volume) * (4.0 * prm.inv_dx * prm.inv_dx) * PF + mass[:, None, None] * C
    mom = mass[:, None, None] * v[:, None, :] + np.einsum("nab,nkb->nka", A, dpos)  # [n,27,3]
    R1 = prm.res + 1
    gv = np.zeros((R1 ** 3, 3))
    gm = np.zeros((R1 ** 3, 1))
    np.add.at(gv, idx.ravel(), (W[..., None] * mom).reshape(-1, 3))
    np.add.at(gm, idx.ravel(), (W * mass[:, None]).reshape(-1, 1))
    vg, keep, has = _grid_masks(gv, gm, prm)
    vgp = vg[idx]  # [n,27,3]
    v1 = np.einsum("nk,nka->na", W, vgp)
    C1 = 4.0 * prm.inv_dx * np.einsum("nk,nka,nkb->nab", W, vgp, rel)
    x1 = x + prm.dt * v1
    F1 = (np.eye(3)[None] + prm.dt * C1) @ F
    out = (x1, v1, F1, C1)
    if not tape:
        return out
    return out, dict(W=W, dW=dW, idx=idx, rel=rel, dpos=dpos, R=R, J=J, A=A, mom=mom, gv=gv, gm=gm,
                     vg=vg, keep=keep, has=has, vgp=vgp, v1=v1, C1=C1, mu=mu, lam=lam)


def _skew(y):
    z = np.zeros(y.shape[:-1] + (3, 3))
    z[..., 0, 1], z[..., 0, 2] = -y[..., 2], y[..., 1]
    z[..., 1, 0], z[..., 1, 2] = y[..., 2], -y[..., 0]
    z[..., 2, 0], z[..., 2, 1] = -y[..., 1], y[..., 0]
    return z


def _cof(F):
    return np.linalg.det(F)[:, None, None] * np.transpose(np.linalg.inv(F), (0, 2, 1))


def polar_vjp(F, R, Rbar):
    """dL/dF of L(R(F)) for the orthogonal polar factor R of F (any sign of det F)."""
    S = np.transpose(R, (0, 2, 1)) @ F
    S = 0.5 * (S + np.transpose(S, (0, 2, 1)))
    M = np.transpose(R, (0, 2, 1)) @ Rbar
    m = np.stack([M[:, 2, 1] - M[:, 1, 2], M[:, 0, 2] - M[:, 2, 0], M[:, 1, 0] - M[:, 0, 1]], axis=1)
    K = np.trace(S, axis1=1, axis2=2)[:, None, None] * np.eye(3)[None] - S
    y = np.linalg.solve(K, m[..., None])[..., 0]
    return R @ _skew(y)


def backward(state, mass, mu0, lam0, prm: Params3D, adj_out):
    """Adjoint of ``forward``: adj_out = (xb, vb, Fb, Cb) of the substep's output; returns the
    adjoints of its input state and the per-particle dL/dmu0, dL/dlam0 of this substep."""
    x, v, F, C = state
    (x1, v1, F1, C1), t = forward(state, mass, mu0, lam0, prm, tape=True)
    xb1, vb1, Fb1, Cb1 = adj_out
    dt, inv_dx = prm.dt, prm.inv_dx
    W, dW, idx, rel, vgp = t["W"], t["dW"], t["idx"], t["rel"], t["vgp"]
    Ft = np.transpose(F, (0, 2, 1))
    # ---- reverse G2P (scatter)
    vbt = vb1 + dt * xb1
    Cbt = Cb1 + dt * Fb1 @ Ft
    Fb = np.transpose(np.eye(3)[None] + dt * C1, (0, 2, 1)) @ Fb1
    node_term = np.einsum("na,nka->nk", vbt, vgp) + 4.0 * inv_dx * np.einsum("nab,nka,nkb->nk", Cbt, vgp, rel)
    xb = xb1 + inv_dx * (np.einsum("nkd,nk->nd", dW, node_term)
                         - 4.0 * inv_dx * np.einsum("nad,na->nd", Cbt, v1))
    vg_bar = np.zeros_like(t["vg"])
    contrib = W[..., None] * (vbt[:, None, :] + 4.0 * inv_dx * np.einsum("nab,nkb->nka", Cbt, rel))
    np.add.at(vg_bar, idx.ravel(), contrib.reshape(-1, 3))
    # ---- reverse grid
    gv, gm, keep, has = t["gv"], t["gm"], t["keep"], t["has"]
    vb_m = np.where(keep, vg_bar, 0.0)
    gv_bar = vb_m.copy()
    gm_bar = np.zeros(gm.shape[0])
    gv_bar[has] = vb_m[has] / gm[has]
    gm_bar[has] = -np.einsum("na,na->n", vb_m[has], gv[has]) / (gm[has, 0] ** 2)
    # ---- reverse P2G (gather)
    gvb = gv_bar[idx]  # [n,27,3]
    gmb = gm_bar[idx]  # [n,27]
    A, mom, dpos, R, J = t["A"], t["mom"], t["dpos"], t["R"], t["J"]
    gsum = np.einsum("nk,nka->na", W, gvb)
    Abar = np.einsum("nk,nka,nkb->nab", W, gvb, dpos)
    term = np.einsum("nka,nka->nk", gvb, mom) + gmb * mass[:, None]
    xb = xb + inv_dx * np.einsum("nkd,nk->nd", dW, term) - np.einsum("nad,na->nd", A, gsum)
    vb = mass[:, None] * gsum
    Cb = mass[:, None, None] * Abar
    G = -(prm.dt * prm.volume) * (4.0 * inv_dx * inv_dx) * Abar
    mu, lam = t["mu"], t["lam"]
    sG = np.trace(G, axis1=1, axis2=2) if prm.lam_diagonal else G.sum(axis=(1, 2))
    Fb = Fb + 2.0 * mu[:, None, None] * (G @ F + np.transpose(G, (0, 2, 1)) @ (F - R))
    Fb = Fb + (lam * (2.0 * J - 1.0) * sG)[:, None, None] * _cof(F)
    Fb = Fb + polar_vjp(F, R, -2.0 * mu[:, None, None] * G @ F)
    mu0b = prm.hardening * 2.0 * np.einsum("nab,nab->n", G, (F - R) @ Ft)
    lam0b = prm.hardening * (J - 1.0) * J * sG
    return (xb, vb, Fb, Cb), mu0b, lam0b


def rollout(state, mass, mu0, lam0, prm: Params3D, steps: int):
    s = state
    for _ in range(steps):
        s = forward(s, mass, mu0, lam0, prm)
    return s


def rollout_backward(state, mass, mu0, lam0, prm: Params3D, steps: int, adj_out):
    """Reverse of ``rollout`` storing every state (small cases only)."""
    states = [state]
    for _ in range(steps):
        states.append(forward(states[-1], mass, mu0, lam0, prm))
    adj = adj_out
    mub = np.zeros_like(mu0)
    lamb = np.zeros_like(lam0)
    for s in reversed(states[:-1]):
        adj, m, l = backward(s, mass, mu0, lam0, prm, adj)
        mub += m
        lamb += l
    return adj, mub, lamb
