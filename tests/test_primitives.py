"""Scene primitives against the reference's own outputs (tests/golden/primitives.npz)."""
import numpy as np

from golden_cases import load
from femflow_gb300.simulation.mpm import primitives as P


def test_grid_matches_reference():
    d = load("primitives")
    np.testing.assert_array_equal(P.grid((3, 4, 2)), d["grid_3_4_2"])
    np.testing.assert_array_equal(P.grid((5, 1, 3)), d["grid_5_1_3"])


def test_implicit_points_of_a_callers_own_function_match_reference():
    """A caller's own implicit function is called point by point, as the reference calls it (the
    reference's three surfaces go to the GPU; tests/test_gpu_primitives.py)."""
    d = load("primitives")
    for fn in ("gyroid", "diamond", "primitive"):
        f = getattr(P, fn)
        own = lambda k, t, pos, f=f: f(k, t, pos)
        np.testing.assert_allclose(P.generate_implicit_points(own, 0.35, 0.15, 12), d[f"{fn}_a"], rtol=0, atol=0)
        np.testing.assert_allclose(P.generate_implicit_points(own, 0.5, -0.3, 9), d[f"{fn}_b"], rtol=0, atol=0)


def test_cube_points_match_reference():
    d = load("primitives")
    np.testing.assert_array_equal(P.generate_cube_points((0.1, 0.4), (0.2, 0.5), (0.3, 0.9), 5), d["cube"])


def test_unknown_implicit_function_raises():
    import pytest
    with pytest.raises(ValueError):
        P.generate_implicit_points("torus", 0.3, 0.1, 4)
