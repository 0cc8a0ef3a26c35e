"""femflow_gb300 — FEMFlow's MLS-MPM substep on GB300 (sm_103a).

Drop-in for ``femflow.solvers.mpm``: the same module layout and call signatures
(``solvers.mpm.mls_mpm.solve_mls_mpm_3d``, ``solvers.mpm.three_d.{p2g,grid_op,g2p}``,
``solvers.mpm.two_d.{p2g,grid_op,g2p}``), computed by hand-written CUDA kernels through the C ABI
of ``include/femflow_mpm.h``.  ``MPMSolver`` is the resident, block-sorted fast path.
"""
from . import _native  # noqa: F401

__version__ = "0.1.0"


def library_path() -> str:
    return _native.LIB_PATH
