"""The FP64 numpy adjoint of the 2D substep (oracle/adjoint2d.py) against its pins (CPU).

* its forward half equals the C oracle's 2D substep (itself pinned to the reference's goldens);
* its reverse half equals FP64 central differences of that forward, for every input of the
  substep (x, v, F, C) and for the Lamé parameters, one substep (by the 0.05 wall band too) and a
  short rollout, and the rotation's derivative on its own.
"""
import numpy as np
import pytest

import oracle as O
from oracle import adjoint2d as A2


def _state(rng, n, lo=0.2, hi=0.8, fstd=0.05):
    x = rng.uniform(lo, hi, (n, 2))
    v = rng.normal(0, 0.3, (n, 2))
    F = np.eye(2)[None] + rng.normal(0, fstd, (n, 2, 2))
    C = rng.normal(0, 1.0, (n, 2, 2))
    return x, v, F, C


def _material(n, mu=400.0, lam=600.0, m=1e-4):
    return np.full(n, m), np.full(n, mu), np.full(n, lam)


@pytest.mark.parametrize("model", ["neo_hookean", "fixed_corotated"])
def test_forward_matches_c_oracle(model):
    rng = np.random.default_rng(0)
    n, res = 500, 32
    prm = A2.Params2D(res=res, dt=2e-4, volume=1e-4, lam_diagonal=model == "fixed_corotated")
    x, v, F, C = _state(rng, n, lo=0.02, hi=0.98)  # the wall band on every side
    mass, mu0, lam0 = _material(n)
    x1, v1, F1, C1 = A2.forward((x, v, F, C), mass, mu0, lam0, prm)
    xc, vc, Fc, Cc, Jp = x.copy(), v.copy(), F.copy(), C.copy(), np.ones((n, 1))
    O.substep_2d(res, float(res), 1.0, 400.0, 600.0, 1e-4, 1 / res, prm.dt, prm.volume, prm.gravity, xc, vc, Fc,
                 Cc, Jp, model=model)
    np.testing.assert_allclose(x1, xc, rtol=0, atol=1e-14)
    np.testing.assert_allclose(v1, vc, rtol=0, atol=1e-13 * np.abs(vc).max())
    np.testing.assert_allclose(C1, Cc, rtol=0, atol=1e-12 * np.abs(Cc).max())
    # the reference's SVD rebuild of F may flip its sign (two_d/g2p.py:37-43); F F^T is what it keeps
    np.testing.assert_allclose(F1 @ np.transpose(F1, (0, 2, 1)), Fc @ np.transpose(Fc, (0, 2, 1)), rtol=0,
                               atol=1e-13)


def _fd_check(loss, st, adj, rng, eps, tol=1e-6):
    for i, name in enumerate("xvFC"):
        d = rng.normal(size=st[i].shape)
        sp, sm = list(st), list(st)
        sp[i] = st[i] + eps[name] * d
        sm[i] = st[i] - eps[name] * d
        fd = (loss(tuple(sp)) - loss(tuple(sm))) / (2 * eps[name])
        an = float((adj[i] * d).sum())
        assert abs(fd - an) <= tol * abs(fd), (name, fd, an)


@pytest.mark.parametrize("seed,fstd,diag,lo,hi", [(1, 0.05, False, 0.2, 0.8), (2, 0.3, False, 0.2, 0.8),
                                                  (6, 0.3, True, 0.2, 0.8), (7, 0.05, False, 0.02, 0.98)])
def test_substep_adjoint_matches_central_differences(seed, fstd, diag, lo, hi):
    rng = np.random.default_rng(seed)
    n, res = 300, 32
    prm = A2.Params2D(res=res, dt=2e-4, volume=1e-4, lam_diagonal=diag)
    st = _state(rng, n, lo=lo, hi=hi, fstd=fstd)
    mass, mu0, lam0 = _material(n)
    if lo < 0.05:
        _, tape = A2.forward(st, mass, mu0, lam0, prm, tape=True)
        assert (~tape["keep"]).any(axis=1).sum() > 0  # some nodes stopped by the band
    wts = [rng.normal(size=a.shape) for a in st]

    def loss(s, m0=mu0, l0=lam0):
        return sum(float((w * o).sum()) for w, o in zip(wts, A2.forward(s, mass, m0, l0, prm)))

    adj, mub, lamb = A2.backward(st, mass, mu0, lam0, prm, tuple(wts))
    _fd_check(loss, st, adj, rng, dict(x=1e-8, v=1e-5, F=1e-6, C=1e-5))
    for g, kw in ((mub, "m0"), (lamb, "l0")):
        base = mu0 if kw == "m0" else lam0
        h = 1e-3
        fd = (loss(st, **{kw: base + h}) - loss(st, **{kw: base - h})) / (2 * h)
        assert abs(fd - g.sum()) <= 1e-6 * abs(fd)


def test_rollout_adjoint_matches_central_differences():
    rng = np.random.default_rng(4)
    n, res, steps = 200, 32, 6
    prm = A2.Params2D(res=res, dt=5e-4, volume=1e-4)
    st = _state(rng, n)
    mass, mu0, lam0 = _material(n)
    wts = [rng.normal(size=a.shape) for a in st]

    def loss(s, m0=mu0, l0=lam0):
        return sum(float((w * o).sum()) for w, o in zip(wts, A2.rollout(s, mass, m0, l0, prm, steps)))

    adj, mub, lamb = A2.rollout_backward(st, mass, mu0, lam0, prm, steps, tuple(wts))
    _fd_check(loss, st, adj, rng, dict(x=1e-8, v=1e-5, F=1e-6, C=1e-5))
    h = 1e-3
    fd = (loss(st, m0=mu0 + h) - loss(st, m0=mu0 - h)) / (2 * h)
    assert abs(fd - mub.sum()) <= 1e-6 * abs(fd)


def test_rotation_vjp():
    rng = np.random.default_rng(5)
    F = np.eye(2)[None] + rng.normal(0, 0.3, (60, 2, 2))
    F[:10, 0] *= -1.0  # reflections too: the closed form still has a derivative
    Rb = rng.normal(size=F.shape)
    g = A2.polar_vjp(F, Rb)
    d = rng.normal(size=F.shape)
    h = 1e-6
    fd = ((A2.polar(F + h * d)[0] * Rb).sum() - (A2.polar(F - h * d)[0] * Rb).sum()) / (2 * h)
    assert abs(fd - (g * d).sum()) <= 1e-7 * abs(fd)
