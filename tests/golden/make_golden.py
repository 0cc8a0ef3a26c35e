"""Generate the golden fixtures in this folder from the unmodified FEMFlow reference solver.

Run once, in a container that holds the reference checkout (it is not available where the GPU
tests run, which is why the outputs are committed):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py <reference checkout>

(or with the checkout's root in the environment variable FEMFLOW_REFERENCE).

numba is not installed, so a no-op ``numba`` module is placed in ``sys.modules`` first: ``njit``,
``jit`` and ``experimental.jitclass`` become identity decorators, ``typed.List`` becomes ``list``.
The reference functions then run unchanged in CPython (float64 numpy).  The ``femflow`` package
object is created by hand so that its ``__init__`` (which imports meshing, GUI and FEM modules
with unavailable dependencies) is not executed; only the solver modules are imported.

Fixtures written:
  kat.npz         known-answer vectors of the reference's own (stale) MPM tests, restated on the
                  current API: B-spline weights (femflow/solvers/mpm/tests/test_utils.py:6-15),
                  2D stress (tests/test_particle_to_grid.py:41-50), the 2D P2G grid
                  (tests/test_particle_to_grid.py:53-80 + tests/ground_truth_grid.txt) and the
                  full 2D step (tests/test_grid_to_particle.py:45-103), each with the current
                  reference output beside the historical expected values.
  ref2d_*.npz     seeded 2D cases run through two_d.p2g / grid_op / g2p.
  ref3d_*.npz     seeded 3D cases run through three_d.p2g / grid_op / g2p and solve_mls_mpm_3d.
  primitives.npz  lattice and scene points of femflow/simulation/mpm/primitives.py.
  colliders.npz   three_d/grid_op.py:50-67 check_collision_points (defined, never called by the
                  reference) on seeded grids and planes, including its literal normal + 1/|normal|.

``--only colliders`` regenerates that fixture alone.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def install_reference(ref_root: str):
    def _ident(*a, **k):
        if len(a) == 1 and callable(a[0]) and not k:
            return a[0]
        return lambda f: f

    class _TypeStub:
        def __getitem__(self, k):
            return self

    nb = types.ModuleType("numba")
    nb.njit = _ident
    nb.jit = _ident
    nb.float64 = _TypeStub()
    exp = types.ModuleType("numba.experimental")
    exp.jitclass = _ident
    nb.experimental = exp
    typed = types.ModuleType("numba.typed")
    typed.List = list
    nb.typed = typed
    sys.modules.update({"numba": nb, "numba.experimental": exp, "numba.typed": typed})
    pkg = types.ModuleType("femflow")
    pkg.__path__ = [os.path.join(ref_root, "femflow")]
    sys.modules["femflow"] = pkg
    sys.dont_write_bytecode = True
    from femflow.solvers.mpm import mls_mpm, particle, three_d, two_d, utils  # noqa: F401
    from femflow.numerics import linear_algebra, fem

    return types.SimpleNamespace(mls_mpm=mls_mpm, particle=particle, three_d=three_d, two_d=two_d,
                                 utils=utils, la=linear_algebra, fem=fem)


def lame(E, nu):
    return E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))


# --------------------------------------------------------------------------- KATs
def make_kat(ref, ref_root):
    out = {}
    # B-spline weights, test_utils.py:6-15 (historical expected values).
    fx = np.array((0.631893, 0.965839))
    out["w_fx"] = fx
    out["w_expected"] = np.array([[0.37680488, 0.14266399], [0.61449724, 0.74883303], [0.00869788, 0.10850299]])
    out["w_ref"] = np.array([0.5 * (1.5 - fx) ** 2, 0.75 - (fx - 1) ** 2, 0.5 * (fx - 0.5) ** 2])  # p2g.py:55

    # Shared parameters of the stale 2D tests, hardening folded to 1 on the current API.
    E, nu = 1e4, 0.2
    mu, lam = lame(E, nu)
    res, dx, dt, grav = 80, 1 / 80, 1e-4, -200.0
    out["kat_params"] = np.array([E, nu, mu, lam, res, dx, dt, grav, 1.0, 1.0, 1.0])  # ..., mass, vol, hardening

    # Stress KAT, test_particle_to_grid.py:41-50.
    F = np.array([[1.0, 0.0], [2.51457e-12, 1.0]])
    C = np.array([[0.0, 0.0], [2.51457e-08, -5.96046e-08]])
    out["stress_F"], out["stress_C"] = F, C
    out["stress_expected"] = np.array([[0, -2.68221e-08], [-1.67638e-09, -5.96046e-08]])
    out["stress_ref"] = ref.utils.fixed_corotated_stress_2d(F, 1 / dx, mu, lam, dt, 1.0, 1.0, C)

    # P2G grid KAT and full-step KAT, three particles.
    x0 = np.array([[0.55, 0.45], [0.45, 0.65], [0.55, 0.85]])
    n = len(x0)
    v = np.zeros((n, 2)); F = np.array([np.eye(2)] * n); C = np.zeros((n, 2, 2)); Jp = np.ones((n, 1))
    gv = np.zeros((res + 1, res + 1, 2)); gm = np.zeros((res + 1, res + 1, 1))
    x = x0.copy()
    ref.two_d.p2g(1 / dx, 1.0, mu, lam, 1.0, dx, dt, 1.0, gv, gm, x, v, F, C, Jp, "neo_hookean")
    out["p2g_x"] = x0
    out["p2g_gv_ref"], out["p2g_gm_ref"] = gv.copy(), gm.copy()
    out["p2g_ground_truth"] = np.loadtxt(os.path.join(ref_root, "femflow/solvers/mpm/tests/ground_truth_grid.txt"))
    ref.two_d.grid_op(res, dt, grav, gv, gm)
    ref.two_d.g2p(1 / dx, dt, gv, x, v, F, C, Jp, "neo_hookean")
    out["step_x_ref"], out["step_v_ref"], out["step_C_ref"], out["step_F_ref"], out["step_Jp_ref"] = x, v, C, F, Jp
    # test_grid_to_particle.py:45-103 historical expected values.
    out["step_x_expected"] = np.array([[0.55, 0.449998], [0.45, 0.649998], [0.55, 0.849998]])
    out["step_v_expected"] = np.array([[0.0, -0.02]] * 3)
    out["step_C_expected"] = np.array([[[0.0, 0.0], [-2.98023e-08, 0.0]]] * 3)
    out["step_F_expected"] = np.array([[[1.0, 0.0], [-2.98023e-12, 1.0]]] * 3)
    np.savez_compressed(os.path.join(HERE, "kat.npz"), **out)


# --------------------------------------------------------------------------- seeded 2D
def random_F(rng, n, dim, stretch=0.05, flip_frac=0.0):
    F = np.zeros((n, dim, dim))
    for p in range(n):
        A = rng.normal(size=(dim, dim))
        Q, Rq = np.linalg.qr(A)
        Q = Q * np.sign(np.diag(Rq))
        if np.linalg.det(Q) < 0:
            Q[:, 0] *= -1
        S = np.eye(dim) + stretch * rng.normal(size=(dim, dim))
        S = 0.5 * (S + S.T)
        F[p] = Q @ S
        if rng.random() < flip_frac:
            F[p][:, 0] *= -1.0  # improper F: the polar factor is a reflection
    return F


def make_2d(ref, name, seed, n, res, E, nu, dt, grav, steps, model="neo_hookean", random_state=False,
            lo=(0.3, 0.4), hi=(0.6, 0.7), hardening=1.0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(lo, hi, size=(n, 2))
    area = (hi[0] - lo[0]) * (hi[1] - lo[1])
    vol = area / n
    mass = 1.0 * vol
    mu, lam = lame(E, nu)
    dx = 1.0 / res
    if random_state:
        v = rng.normal(0, 0.5, size=(n, 2))
        F = random_F(rng, n, 2, 0.05, 0.0)
        C = rng.normal(0, 2.0, size=(n, 2, 2))
        Jp = rng.uniform(0.8, 1.2, size=(n, 1))
    else:
        v = np.zeros((n, 2)); F = np.array([np.eye(2)] * n); C = np.zeros((n, 2, 2)); Jp = np.ones((n, 1))
    out = dict(x0=x.copy(), v0=v.copy(), F0=F.copy(), C0=C.copy(), Jp0=Jp.copy(),
               params=np.array([res, dx, 1 / dx, dt, grav, vol, mass, mu, lam, hardening, steps]),
               model=np.array(model))
    # Phase outputs of the first substep (per-phase parity), then `steps` full substeps.
    for s in range(steps):
        gv = np.zeros((res + 1, res + 1, 2)); gm = np.zeros((res + 1, res + 1, 1))
        ref.two_d.p2g(1 / dx, hardening, mu, lam, mass, dx, dt, vol, gv, gm, x, v, F, C, Jp, model)
        if s == 0:
            out["p2g_gv"], out["p2g_gm"] = gv.copy(), gm.copy()
        ref.two_d.grid_op(res, dt, grav, gv, gm)
        if s == 0:
            out["grid_gv"] = gv.copy()
        ref.two_d.g2p(1 / dx, dt, gv, x, v, F, C, Jp, model)
        if s == 0:
            out.update(g2p_x=x.copy(), g2p_v=v.copy(), g2p_F=F.copy(), g2p_C=C.copy(), g2p_Jp=Jp.copy())
    out.update(x=x, v=v, F=F, C=C, Jp=Jp)
    np.savez_compressed(os.path.join(HERE, f"ref2d_{name}.npz"), **out)


# --------------------------------------------------------------------------- seeded 3D
def make_3d(ref, name, seed, n, res, dt, grav, steps, E_range=(1e3, 1e3), nu=0.3, random_state=False,
            lo=0.3, hi=0.7, hardening=1.0, vel=0.0, flip_frac=0.0, model="neo_hookean"):
    rng = np.random.default_rng(seed)
    x = rng.uniform(lo, hi, size=(n, 3))
    vol = (hi - lo) ** 3 / n
    E = np.exp(rng.uniform(np.log(E_range[0]), np.log(E_range[1]), size=n))
    mass = vol * rng.uniform(0.5, 2.0, size=n)
    mu, lam = lame(E, nu)
    dx = 1.0 / res
    if random_state:
        v = rng.normal(0, vel if vel > 0 else 0.3, size=(n, 3))
        F = random_F(rng, n, 3, 0.05, flip_frac)
        C = rng.normal(0, 2.0, size=(n, 3, 3))
        Jp = rng.uniform(0.8, 1.2, size=(n, 1))
    else:
        v = np.tile(np.array([vel, 0.0, 0.0]), (n, 1))
        F = np.array([np.eye(3)] * n); C = np.zeros((n, 3, 3)); Jp = np.ones((n, 1))
    P = ref.particle.Particle
    particles = [P(x[p].astype(np.float64).copy(), 0.0, float(mass[p]), float(lam[p]), float(mu[p])) for p in range(n)]
    out = dict(x0=x.copy(), mass=mass, mu0=mu, lam0=lam, v0=v.copy(), F0=F.copy(), C0=C.copy(), Jp0=Jp.copy(),
               params=np.array([res, dx, 1 / dx, dt, grav, vol, hardening, steps]), model=np.array(model))
    R = res + 1
    # First substep phase by phase (per-phase API parity) ...
    gv = np.zeros((R, R, R, 3)); gm = np.zeros((R, R, R, 1))
    ref.three_d.p2g(1 / dx, hardening, dx, dt, vol, gv, gm, particles, v, F, C, Jp, model)
    out["p2g_gv"], out["p2g_gm"] = gv.copy(), gm.copy()
    ref.three_d.grid_op(res, dx, dt, grav, gv, gm)
    out["grid_gv"] = gv.copy()
    ref.three_d.g2p(1 / dx, dt, gv, particles, v, F, C, Jp, model)
    pos = np.array([p.pos for p in particles])
    out.update(g2p_x=pos.copy(), g2p_v=v.copy(), g2p_F=F.copy(), g2p_C=C.copy(), g2p_Jp=Jp.copy())
    # ... then the remaining substeps through the reference driver function.
    if model == "neo_hookean":
        for _ in range(steps - 1):
            ref.mls_mpm.solve_mls_mpm_3d(res, 1 / dx, hardening, dx, dt, vol, grav, particles, v, F, C, Jp)
    pos = np.array([p.pos for p in particles])
    out.update(x=pos, v=v, F=F, C=C, Jp=Jp)
    np.savez_compressed(os.path.join(HERE, f"ref3d_{name}.npz"), **out)


def make_primitives(ref_root):
    """Scene primitives (femflow/simulation/mpm/primitives.py).  numerics/geometry.py imports igl
    and wildmeshing at module level; neither is used by grid(), so empty modules stand in."""
    import importlib.util

    for name in ("igl", "wildmeshing"):
        sys.modules.setdefault(name, types.ModuleType(name))
    spec = importlib.util.spec_from_file_location(
        "ref_primitives", os.path.join(ref_root, "femflow/simulation/mpm/primitives.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    from femflow.numerics.geometry import grid

    out = {"grid_3_4_2": grid(np.array((3, 4, 2))), "grid_5_1_3": grid(np.array((5, 1, 3)))}
    for fn in ("gyroid", "diamond", "primitive"):
        out[f"{fn}_a"] = m.generate_implicit_points(fn, 0.35, 0.15, 12)
        out[f"{fn}_b"] = m.generate_implicit_points(fn, 0.5, -0.3, 9)
    out["cube"] = m.generate_cube_points((0.1, 0.4), (0.2, 0.5), (0.3, 0.9), 5)
    np.savez_compressed(os.path.join(HERE, "primitives.npz"), **out)


def make_colliders(ref):
    """check_collision_points on two seeded 13^3 grids with three seeded planes each."""
    import importlib

    # the module (three_d/__init__.py re-exports the grid_op function under the same name)
    ref_grid_op = importlib.import_module("femflow.solvers.mpm.three_d.grid_op")

    out = {}
    for case, seed in (("a", 0), ("b", 1)):
        rng = np.random.default_rng(100 + seed)
        res, dx = 12, 1.0 / 12
        gv = rng.normal(0.0, 1.0, (res + 1, res + 1, res + 1, 3))
        points = rng.uniform(0.2, 0.8, (3, 3))
        normals = rng.normal(0.0, 1.0, (3, 3))
        got = gv.copy()
        ref_grid_op.check_collision_points(points, normals, res, dx, got)
        out.update({f"{case}_res": res, f"{case}_dx": dx, f"{case}_points": points, f"{case}_normals": normals,
                    f"{case}_grid_in": gv, f"{case}_grid_out": got})
    np.savez_compressed(os.path.join(HERE, "colliders.npz"), **out)


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if "--only" in sys.argv and args and args[0] == sys.argv[sys.argv.index("--only") + 1]:
        args = args[1:]
    ref_root = args[0] if args else os.environ.get("FEMFLOW_REFERENCE")
    if not ref_root:
        sys.exit("usage: make_golden.py <reference checkout> [--only colliders] "
                 "(or set FEMFLOW_REFERENCE to the checkout's root)")
    ref = install_reference(ref_root)
    if "--only" in sys.argv:
        only = sys.argv[sys.argv.index("--only") + 1]
        {"colliders": lambda: make_colliders(ref)}[only]()
        print(f"{only} fixture written to", HERE)
        return
    make_colliders(ref)
    make_primitives(ref_root)
    make_kat(ref, ref_root)
    # C1-like scene (block in [0.3,0.6]x[0.4,0.7], rho=1, E=1e4, nu=0.2) at reduced N/res.
    make_2d(ref, "c1_small", seed=0, n=256, res=32, E=1e4, nu=0.2, dt=1e-4, grav=-9.8, steps=6)
    make_2d(ref, "random_state", seed=1, n=200, res=24, E=5e3, nu=0.3, dt=1e-4, grav=-9.8, steps=3,
            random_state=True)
    make_2d(ref, "snow", seed=2, n=200, res=24, E=5e3, nu=0.3, dt=1e-4, grav=-9.8, steps=3, model="snow",
            random_state=True, hardening=10.0)
    make_2d(ref, "walls", seed=3, n=150, res=20, E=2e3, nu=0.25, dt=2e-4, grav=-50.0, steps=4,
            random_state=True, lo=(0.04, 0.03), hi=(0.93, 0.93))
    # 3D: C2-like two-cube-free small scene, random state with improper F, near-wall clamp case.
    make_3d(ref, "drop_small", seed=0, n=160, res=16, dt=1e-4, grav=-9.8, steps=4, E_range=(2e3, 2e3))
    make_3d(ref, "random_state", seed=1, n=120, res=12, dt=1e-4, grav=-9.8, steps=3, E_range=(1e3, 1e4),
            random_state=True, flip_frac=0.1)
    make_3d(ref, "walls_clamp", seed=2, n=120, res=12, dt=5e-3, grav=-30.0, steps=3, E_range=(50, 200),
            random_state=True, lo=0.12, hi=0.88, vel=6.0)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
