"""GPU scene sampling (ffmpm_implicit_points) against the reference's generate_implicit_points.

The reference (femflow/simulation/mpm/primitives.py:46-61) evaluates a triply periodic surface at
every point of a res^3 lattice and keeps the points with ``inside > t`` in lattice order.  The
kernel must return the same points in the same order: bit for bit on the reference's own outputs
(tests/golden/primitives.npz), and at larger lattices the same set as a float64 numpy evaluation,
except for points whose value lies within rounding of the threshold (where two sine libraries
may disagree in the last bit).
"""
import numpy as np
import pytest

from golden_cases import load
from femflow_gb300.simulation.mpm import primitives as P

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fn", ["gyroid", "diamond", "primitive"])
def test_gpu_implicit_points_equal_reference_outputs(fn):
    d = load("primitives")
    np.testing.assert_array_equal(P.generate_implicit_points(fn, 0.35, 0.15, 12), d[f"{fn}_a"])
    np.testing.assert_array_equal(P.generate_implicit_points(fn, 0.5, -0.3, 9), d[f"{fn}_b"])
    # the module's functions themselves take the same path
    np.testing.assert_array_equal(P.generate_implicit_points(getattr(P, fn), 0.35, 0.15, 12), d[f"{fn}_a"])


@pytest.mark.parametrize("fn,k,t,res", [("gyroid", 0.3, 0.2, 64), ("diamond", 0.25, -0.1, 97), ("primitive", 0.4, 0.5, 128),
                                        ("gyroid", 1.0, 0.0, 1), ("primitive", 0.7, -3.5, 5)])
def test_gpu_implicit_points_equal_numpy_evaluation(fn, k, t, res):
    g = P.grid((res, res, res))
    val = np.asarray(getattr(P, fn)(k, t, g))
    want_mask = val > t
    got = P.implicit_points_gpu(fn, k, t, res).cpu().numpy()
    if len(got) == int(want_mask.sum()) and np.array_equal(got, g[want_mask]):
        return
    # any difference must come from points within rounding of the threshold, and the order is
    # lattice order either way
    idx = np.lexsort((got[:, 0], got[:, 1], got[:, 2]))
    assert np.array_equal(idx, np.arange(len(got)))
    got_set = {tuple(r) for r in got}
    want_set = {tuple(r) for r in g[want_mask]}
    diff = got_set ^ want_set
    near = {tuple(r) for r, v in zip(g, val) if abs(v - t) < 1e-12}
    assert diff <= near, len(diff - near)
