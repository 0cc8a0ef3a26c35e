"""FP64 numpy restatement of the 2D MLS-MPM substep and of its adjoint — test infrastructure only.

The forward half restates the reference's 2D substep (femflow/solvers/mpm/two_d/p2g.py:11-76,
grid_op.py:5-24, g2p.py:5-47) for the elastic models, vectorised over particles:

* P2G    two_d/p2g.py:40-76      base = trunc(x*inv_dx - 0.5), quadratic B-spline weights,
                                   A = -dt*vol*4*inv_dx^2*PF + m*C with
                                   PF = 2mu(F-R)F^T + lam(J-1)J on all four entries (utils.py:52-92)
                                   or, with ``lam_diagonal``, on the diagonal only (model
                                   "fixed_corotated"), R the closed-form rotation of
                                   linear_algebra.py:97-116 (with its +1e-10)
* grid   two_d/grid_op.py:5-24   on nodes with mass: v = p/m, v_y += dt*g, then the 0.05 wall band:
                                   x < 0.05, x > 0.95 or y > 0.95 stop the node, y < 0.05 keeps only
                                   v_y > 0 (x = i/res, y = j/res); no velocity clamp in 2D
* G2P    two_d/g2p.py:21-46      v, C = 4*inv_dx*sum w*v_i (x) (i - fx), x += dt*v,
                                   F <- (I + dt*C) F (the SVD rebuild of g2p.py:37-43 returns F
                                   itself up to the sign of LAPACK's factors, which no observable
                                   sees); Jp does not feed back for the elastic models

It is pinned to the C oracle (``oracle.substep_2d``), itself pinned to the reference's golden
vectors.  The reverse half is the exact derivative of this forward, derived by hand like the 3D
one (oracle/adjoint3d.py): reverse G2P scatters to the grid, reverse grid applies the wall masks
and the division by mass, reverse P2G gathers; the rotation's derivative follows from
c = x/d, s = y/d, d = |(x, y)| + 1e-10 with x = F00 + F11, y = F10 - F01.  It is pinned by central
finite differences of the forward (tests/test_adjoint_oracle.py).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

OFFS = np.array([(i, j) for i in range(3) for j in range(3)], dtype=np.int64)  # [9,2]


@dataclass
class Params2D:
    res: int
    dt: float
    volume: float
    gravity: float = -9.8
    hardening: float = 1.0
    # False: the reference's stress, lam(J-1)J added to all four entries of PF (utils.py:87);
    # True: the textbook fixed-corotated stress, lam(J-1)J on the diagonal only
    lam_diagonal: bool = False

    @property
    def dx(self) -> float:
        return 1.0 / self.res

    @property
    def inv_dx(self) -> float:
        return float(self.res)


def _weights(fx):
    w = np.stack([0.5 * (1.5 - fx) ** 2, 0.75 - (fx - 1.0) ** 2, 0.5 * (fx - 0.5) ** 2], axis=1)
    dw = np.stack([fx - 1.5, -2.0 * (fx - 1.0), fx - 0.5], axis=1)
    return w, dw


def _stencil(x, prm):
    base = (x * prm.inv_dx - 0.5).astype(np.int64)
    if (base < 0).any() or (base + 2 > prm.res).any():
        raise RuntimeError("particle out of grid bounds")
    fx = x * prm.inv_dx - base
    w, dw = _weights(fx)
    a, b = OFFS[:, 0], OFFS[:, 1]
    W = w[:, a, 0] * w[:, b, 1]  # [n,9]
    dW = np.stack([dw[:, a, 0] * w[:, b, 1], w[:, a, 0] * dw[:, b, 1]], axis=2)  # [n,9,2] d/dfx
    R1 = prm.res + 1
    node = base[:, None, :] + OFFS[None]
    idx = node[..., 0] * R1 + node[..., 1]  # [n,9]
    rel = OFFS[None].astype(np.float64) - fx[:, None, :]
    return W, dW, idx, rel


def polar(F):
    """The reference's 2D rotation (linear_algebra.py:97-116), batched: returns R and (x, y, d)."""
    x = F[:, 0, 0] + F[:, 1, 1]
    y = F[:, 1, 0] - F[:, 0, 1]
    d = np.sqrt(x * x + y * y) + 1e-10
    c, s = x / d, y / d
    R = np.stack([np.stack([c, -s], axis=1), np.stack([s, c], axis=1)], axis=1)
    return R, (x, y, d)


def polar_vjp(F, Rbar):
    """dL/dF of L(R(F)) for the closed-form rotation above, +1e-10 included."""
    _, (x, y, d) = polar(F)
    r = d - 1e-10
    cb = Rbar[:, 0, 0] + Rbar[:, 1, 1]
    sb = Rbar[:, 1, 0] - Rbar[:, 0, 1]
    k = 1.0 / (r * d * d)
    dcx, dcy = 1.0 / d - x * x * k, -x * y * k
    dsx, dsy = -x * y * k, 1.0 / d - y * y * k
    xb = cb * dcx + sb * dsx
    yb = cb * dcy + sb * dsy
    G = np.zeros_like(F)
    G[:, 0, 0] = xb
    G[:, 1, 1] = xb
    G[:, 1, 0] = yb
    G[:, 0, 1] = -yb
    return G


def _grid(gv, gm, prm):
    """Grid rule of two_d/grid_op.py and the per-component pass-through mask of its derivative."""
    R1 = prm.res + 1
    I = np.stack(np.unravel_index(np.arange(R1 * R1), (R1, R1)), axis=1)
    has = gm[:, 0] > 0
    v = gv.copy()
    v[has] /= gm[has]
    v[has, 1] += prm.dt * prm.gravity
    xs, ys = I[:, 0] / prm.res, I[:, 1] / prm.res
    stop = has & ((xs < 0.05) | (xs > 1 - 0.05) | (ys > 1 - 0.05))
    v[stop] = 0.0
    low = has & (ys < 0.05)
    neg = low & ~(v[:, 1] > 0.0)
    v[neg, 1] = 0.0
    keep = np.ones_like(v, dtype=bool)
    keep[stop] = False
    keep[neg, 1] = False
    return v, keep, has


def forward(state, mass, mu0, lam0, prm: Params2D, tape: bool = False):
    """One substep.  state = (x[n,2], v[n,2], F[n,2,2], C[n,2,2]); mass/mu0/lam0 are [n] arrays."""
    x, v, F, C = state
    W, dW, idx, rel = _stencil(x, prm)
    dpos = rel * prm.dx
    mu = mu0 * prm.hardening
    lam = lam0 * prm.hardening
    R, _ = polar(F)
    J = np.linalg.det(F)
    PF = 2.0 * mu[:, None, None] * (F - R) @ np.transpose(F, (0, 2, 1)) + \
        (lam * (J - 1.0) * J)[:, None, None] * (np.eye(2)[None] if prm.lam_diagonal else 1.0)
    A = -(prm.dt * prm.volume) * (4.0 * prm.inv_dx * prm.inv_dx) * PF + mass[:, None, None] * C
    mom = mass[:, None, None] * v[:, None, :] + np.einsum("nab,nkb->nka", A, dpos)  # [n,9,2]
    R1 = prm.res + 1
    gv = np.zeros((R1 * R1, 2))
    gm = np.zeros((R1 * R1, 1))
    np.add.at(gv, idx.ravel(), (W[..., None] * mom).reshape(-1, 2))
    np.add.at(gm, idx.ravel(), (W * mass[:, None]).reshape(-1, 1))
    vg, keep, has = _grid(gv, gm, prm)
    vgp = vg[idx]
    v1 = np.einsum("nk,nka->na", W, vgp)
    C1 = 4.0 * prm.inv_dx * np.einsum("nk,nka,nkb->nab", W, vgp, rel)
    x1 = x + prm.dt * v1
    F1 = (np.eye(2)[None] + prm.dt * C1) @ F
    out = (x1, v1, F1, C1)
    if not tape:
        return out
    return out, dict(W=W, dW=dW, idx=idx, rel=rel, dpos=dpos, R=R, J=J, A=A, mom=mom, gv=gv, gm=gm,
                     vg=vg, keep=keep, has=has, vgp=vgp, v1=v1, C1=C1, mu=mu, lam=lam)


def _cof(F):
    """d det F / dF = [[F11, -F10], [-F01, F00]]."""
    return np.stack([np.stack([F[:, 1, 1], -F[:, 1, 0]], axis=1), np.stack([-F[:, 0, 1], F[:, 0, 0]], axis=1)], axis=1)


def backward(state, mass, mu0, lam0, prm: Params2D, adj_out):
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
    Fb = np.transpose(np.eye(2)[None] + dt * C1, (0, 2, 1)) @ Fb1
    node_term = np.einsum("na,nka->nk", vbt, vgp) + 4.0 * inv_dx * np.einsum("nab,nka,nkb->nk", Cbt, vgp, rel)
    xb = xb1 + inv_dx * (np.einsum("nkd,nk->nd", dW, node_term)
                         - 4.0 * inv_dx * np.einsum("nad,na->nd", Cbt, v1))
    vg_bar = np.zeros_like(t["vg"])
    contrib = W[..., None] * (vbt[:, None, :] + 4.0 * inv_dx * np.einsum("nab,nkb->nka", Cbt, rel))
    np.add.at(vg_bar, idx.ravel(), contrib.reshape(-1, 2))
    # ---- reverse grid
    gv, gm, keep, has = t["gv"], t["gm"], t["keep"], t["has"]
    vb_m = np.where(keep, vg_bar, 0.0)
    gv_bar = vb_m.copy()
    gm_bar = np.zeros(gm.shape[0])
    gv_bar[has] = vb_m[has] / gm[has]
    gm_bar[has] = -np.einsum("na,na->n", vb_m[has], gv[has]) / (gm[has, 0] ** 2)
    # ---- reverse P2G (gather)
    gvb = gv_bar[idx]
    gmb = gm_bar[idx]
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
    Fb = Fb + polar_vjp(F, -2.0 * mu[:, None, None] * G @ F)
    mu0b = prm.hardening * 2.0 * np.einsum("nab,nab->n", G, (F - R) @ Ft)
    lam0b = prm.hardening * (J - 1.0) * J * sG
    return (xb, vb, Fb, Cb), mu0b, lam0b


def rollout(state, mass, mu0, lam0, prm: Params2D, steps: int):
    s = state
    for _ in range(steps):
        s = forward(s, mass, mu0, lam0, prm)
    return s


def rollout_backward(state, mass, mu0, lam0, prm: Params2D, steps: int, adj_out):
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
