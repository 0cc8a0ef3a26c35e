"""Shared helpers of the GPU parity tests."""
import numpy as np
import torch

# Tolerances of the GPU path against float64 references (oracle / reference golden vectors).
# float64: the same formulas in the same precision, so differences are summation-order rounding.
# float32: the product precision; bounds are a few hundred float32 ulps of each quantity's scale.
TOL = {
    torch.float64: dict(grid=1e-11, x=1e-12, v=1e-10, C=1e-9, F=1e-11, Jp=1e-12),
    torch.float32: dict(grid=2e-5, x=2e-6, v=2e-4, C=2e-3, F=2e-5, Jp=1e-6),
}


def t(a, dtype, device="cuda"):
    return torch.tensor(np.asarray(a), dtype=dtype, device=device)


def n(x):
    return x.detach().double().cpu().numpy()


def close(got, want, rel, scale=None, what=""):
    """max |got - want| <= rel * scale (scale defaults to max |want|, at least 1e-30)."""
    got, want = np.asarray(got, dtype=np.float64), np.asarray(want, dtype=np.float64)
    assert got.shape == want.shape, (what, got.shape, want.shape)
    s = float(np.abs(want).max()) if scale is None else float(scale)
    err = float(np.abs(got - want).max()) if got.size else 0.0
    assert err <= rel * max(s, 1e-30), f"{what}: max err {err:.3e} > {rel:.1e} * {s:.3e}"
    return err


def sign_align(F, Fref):
    s = np.sign(np.einsum("nij,nij->n", F, Fref))[:, None, None]
    s[s == 0] = 1
    return F * s
