"""The corrector network's numpy oracle (oracle/mlp.py), CPU only: bf16 rounding and its exact
(float64) gradient against central differences."""
import numpy as np
import torch

from oracle import mlp as M


def _params(rng):
    P = np.zeros(M.NPARAMS)
    P[0:64 * 128].reshape(64, 128)[:, :102] = rng.normal(0, 0.15, (64, 102))
    for k, n, sd in (("W2", 4096, .18), ("W3", 4096, .18), ("W4", 768, .1), ("b1", 64, .1), ("b2", 64, .1),
                     ("b3", 64, .1), ("b4", 12, .1)):
        P[M.OFF[k]:M.OFF[k] + n] = rng.normal(0, sd, n)
    return P


def test_bf16_rounding_matches_torch():
    x = np.random.default_rng(0).normal(0, 3, 10000).astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).float().numpy()
    np.testing.assert_array_equal(M.bf16(x), ref.astype(np.float64))


def test_exact_gradient_matches_central_differences():
    rng = np.random.default_rng(1)
    P = _params(rng)
    X = np.zeros((64, 128))
    X[:, :102] = rng.normal(0, 1, (64, 102))
    X = M.bf16(X)
    T = rng.normal(0, 1, (64, 12))
    w = rng.uniform(0.5, 2, 12)
    _, g, _ = M.backward(P, X, T, w, exact=True)

    def L(P):
        return float((w * (M.forward_fp64(P, X) - T) ** 2).sum() / 64)

    for k, n in (("W1", 64 * 128), ("W2", 4096), ("W4", 768), ("b1", 64), ("b4", 12)):
        d = np.zeros(M.NPARAMS)
        d[M.OFF[k]:M.OFF[k] + n] = rng.normal(size=n)
        if k == "W1":
            d[0:64 * 128].reshape(64, 128)[:, 102:] = 0
        h = 1e-6
        fd = (L(P + h * d) - L(P - h * d)) / (2 * h)
        assert abs(fd - (g * d).sum()) <= 1e-7 * abs(fd), k


def test_bf16_gradient_close_to_exact():
    rng = np.random.default_rng(2)
    P = _params(rng)
    X = np.zeros((256, 128))
    X[:, :102] = rng.normal(0, 1, (256, 102))
    X = M.bf16(X)
    T = rng.normal(0, 1, (256, 12))
    w = np.ones(12)
    _, g, _ = M.backward(P, X, T, w)
    _, ge, _ = M.backward(P, X, T, w, exact=True)
    assert np.linalg.norm(g - ge) <= 2e-2 * np.linalg.norm(ge)
