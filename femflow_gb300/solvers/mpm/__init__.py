"""Mirror of ``femflow.solvers.mpm`` (femflow/solvers/mpm/__init__.py) on the GPU."""
from . import mls_mpm, particle, three_d, two_d, utils  # noqa: F401
