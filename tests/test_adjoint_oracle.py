"""The FP64 numpy adjoint of the 3D substep (oracle/adjoint3d.py) against its pins (CPU).

* its forward half equals the C oracle's substep (itself pinned to the reference's goldens);
* its reverse half equals FP64 central differences of that forward, for every input of the
  substep (x, v, F, C) and for the Lamé parameters, one substep and a short rollout;
* the C-ABI rejects what the adjoint does not cover (snow, other dims) without touching a GPU.
"""
import ctypes
import os

import numpy as np
import pytest

import oracle as O
from oracle import adjoint3d as A3


def _state(rng, n, lo=0.3, hi=0.7, fstd=0.05):
    x = rng.uniform(lo, hi, (n, 3))
    v = rng.normal(0, 0.3, (n, 3))
    F = np.eye(3)[None] + rng.normal(0, fstd, (n, 3, 3))
    C = rng.normal(0, 1.0, (n, 3, 3))
    return x, v, F, C


def _material(n, mu=400.0, lam=600.0, m=1e-5):
    return np.full(n, m), np.full(n, mu), np.full(n, lam)


@pytest.mark.parametrize("model", ["neo_hookean", "fixed_corotated"])
def test_forward_matches_c_oracle(model):
    rng = np.random.default_rng(0)
    n, res = 400, 16
    prm = A3.Params3D(res=res, dt=2e-4, volume=1e-5, lam_diagonal=model == "fixed_corotated")
    x, v, F, C = _state(rng, n)
    mass, mu0, lam0 = _material(n)
    x1, v1, F1, C1 = A3.forward((x, v, F, C), mass, mu0, lam0, prm)
    xc, vc, Fc, Cc, Jp = x.copy(), v.copy(), F.copy(), C.copy(), np.ones((n, 1))
    O.substep_3d(res, float(res), 1.0, 1 / res, prm.dt, prm.volume, prm.gravity, xc, mass.copy(), mu0.copy(),
                 lam0.copy(), vc, Fc, Cc, Jp, model=model)
    np.testing.assert_allclose(x1, xc, rtol=0, atol=1e-14)
    np.testing.assert_allclose(v1, vc, rtol=0, atol=1e-13 * np.abs(vc).max())
    np.testing.assert_allclose(F1, Fc, rtol=0, atol=1e-13)
    np.testing.assert_allclose(C1, Cc, rtol=0, atol=1e-12 * np.abs(Cc).max())


def _fd_check(loss, st, adj, rng, eps):
    for i, name in enumerate("xvFC"):
        d = rng.normal(size=st[i].shape)
        sp, sm = list(st), list(st)
        sp[i] = st[i] + eps[name] * d
        sm[i] = st[i] - eps[name] * d
        fd = (loss(tuple(sp)) - loss(tuple(sm))) / (2 * eps[name])
        an = float((adj[i] * d).sum())
        assert abs(fd - an) <= 1e-6 * abs(fd), (name, fd, an)


@pytest.mark.parametrize("seed,fstd,diag", [(1, 0.05, False), (2, 0.3, False), (6, 0.3, True)])
def test_substep_adjoint_matches_central_differences(seed, fstd, diag):
    rng = np.random.default_rng(seed)
    n, res = 300, 16
    prm = A3.Params3D(res=res, dt=2e-4, volume=1e-5, lam_diagonal=diag)
    st = _state(rng, n, fstd=fstd)
    mass, mu0, lam0 = _material(n)
    wts = [rng.normal(size=a.shape) for a in st]

    def loss(s, m0=mu0, l0=lam0):
        return sum(float((w * o).sum()) for w, o in zip(wts, A3.forward(s, mass, m0, l0, prm)))

    adj, mub, lamb = A3.backward(st, mass, mu0, lam0, prm, tuple(wts))
    _fd_check(loss, st, adj, rng, dict(x=1e-7, v=1e-5, F=1e-6, C=1e-5))
    for g, kw in ((mub, "m0"), (lamb, "l0")):
        base = mu0 if kw == "m0" else lam0
        h = 1e-3
        fd = (loss(st, **{kw: base + h}) - loss(st, **{kw: base - h})) / (2 * h)
        assert abs(fd - g.sum()) <= 1e-6 * abs(fd)


def test_clamp_and_walls_pass_no_gradient():
    """Particles by the wall band and a grid velocity above the clamp: still exact derivatives."""
    rng = np.random.default_rng(3)
    n, res = 200, 16
    prm = A3.Params3D(res=res, dt=2e-3, volume=1e-5)
    x = rng.uniform(0.04, 0.25, (n, 3))  # inside and next to the 1-cell wall band
    v = rng.normal(0, 3.0, (n, 3))       # 0.9 dx / dt = 28 m/s; momentum kicks push some nodes over it
    v[:20] *= 20.0
    F = np.eye(3)[None] + rng.normal(0, 0.05, (n, 3, 3))
    C = rng.normal(0, 1.0, (n, 3, 3))
    st = (x, v, F, C)
    mass, mu0, lam0 = _material(n)
    (out, tape) = A3.forward(st, mass, mu0, lam0, prm, tape=True)
    assert (~tape["keep"]).any(axis=1).sum() > 0
    wts = [rng.normal(size=a.shape) for a in st]

    def loss(s):
        return sum(float((w * o).sum()) for w, o in zip(wts, A3.forward(s, mass, mu0, lam0, prm)))

    adj, _, _ = A3.backward(st, mass, mu0, lam0, prm, tuple(wts))
    _fd_check(loss, st, adj, rng, dict(x=1e-8, v=1e-5, F=1e-6, C=1e-5))


def test_rollout_adjoint_matches_central_differences():
    rng = np.random.default_rng(4)
    n, res, steps = 200, 16, 6
    prm = A3.Params3D(res=res, dt=5e-4, volume=1e-5)
    st = _state(rng, n)
    mass, mu0, lam0 = _material(n)
    wts = [rng.normal(size=a.shape) for a in st]

    def loss(s, m0=mu0, l0=lam0):
        return sum(float((w * o).sum()) for w, o in zip(wts, A3.rollout(s, mass, m0, l0, prm, steps)))

    adj, mub, lamb = A3.rollout_backward(st, mass, mu0, lam0, prm, steps, tuple(wts))
    _fd_check(loss, st, adj, rng, dict(x=1e-7, v=1e-5, F=1e-6, C=1e-5))
    h = 1e-3
    fd = (loss(st, m0=mu0 + h) - loss(st, m0=mu0 - h)) / (2 * h)
    assert abs(fd - mub.sum()) <= 1e-6 * abs(fd)


def test_polar_vjp_improper_rotation():
    """det F < 0: the reference's R = U Vh is a reflection; its derivative is still exact."""
    rng = np.random.default_rng(5)
    F = np.eye(3)[None] + rng.normal(0, 0.2, (50, 3, 3))
    F[:, 0] *= -1.0
    assert (np.linalg.det(F) < 0).all()
    Rb = rng.normal(size=F.shape)
    R = A3._polar(F)
    g = A3.polar_vjp(F, R, Rb)
    d = rng.normal(size=F.shape)
    h = 1e-6
    fd = ((A3._polar(F + h * d) * Rb).sum() - (A3._polar(F - h * d) * Rb).sum()) / (2 * h)
    assert abs(fd - (g * d).sum()) <= 1e-7 * abs(fd)


def test_capi_rejects_unsupported_adjoints():
    from femflow_gb300 import _native as N
    if not os.path.exists(N.LIB_PATH):
        pytest.skip("library not built")
    lib = N.load()
    p = N.Params(dim=4, res=32, real_bytes=4, dx=1 / 32, inv_dx=32.0, dt=1e-4, volume=1.0, hardening=1.0)
    out = ctypes.c_size_t(0)
    assert lib.ffmpm_adjoint_workspace_size(ctypes.byref(p), 10, ctypes.byref(out)) == N.ERR_UNSUPPORTED
    P, A = N.Particles(), N.Adjoint()
    assert lib.ffmpm_substep_adjoint(ctypes.byref(p), ctypes.byref(P), ctypes.byref(A), None, 0, None) == \
        N.ERR_UNSUPPORTED
    p.dim = 2  # 2D elastic: three (res+1)^2 grids of 32-byte nodes
    assert lib.ffmpm_adjoint_workspace_size(ctypes.byref(p), 10, ctypes.byref(out)) == N.OK
    assert out.value >= 256 + 3 * 32 * 33 ** 2
    assert lib.ffmpm_substep_adjoint(ctypes.byref(p), ctypes.byref(P), ctypes.byref(A), None, 0, None) == \
        N.ERR_WORKSPACE
    p.model = N.MODELS["snow"]
    assert lib.ffmpm_substep_adjoint(ctypes.byref(p), ctypes.byref(P), ctypes.byref(A), None, 0, None) == \
        N.ERR_UNSUPPORTED
    p.dim, p.model = 3, N.MODELS["snow"]
    assert lib.ffmpm_substep_adjoint(ctypes.byref(p), ctypes.byref(P), ctypes.byref(A), None, 0, None) == \
        N.ERR_UNSUPPORTED
    p.model = 9
    assert lib.ffmpm_substep_adjoint(ctypes.byref(p), ctypes.byref(P), ctypes.byref(A), None, 0, None) == \
        N.ERR_UNSUPPORTED
    p.model = N.MODELS["fixed_corotated"]
    assert lib.ffmpm_adjoint_workspace_size(ctypes.byref(p), 10, ctypes.byref(out)) == N.OK
    assert out.value >= 256 + 3 * 32 * 33 ** 3
    assert lib.ffmpm_substep_adjoint(ctypes.byref(p), ctypes.byref(P), ctypes.byref(A), None, 0, None) == \
        N.ERR_WORKSPACE
