"""Mirror of ``femflow.simulation.mpm``: the MPM simulation driver and its scene primitives."""
from . import primitives, simulation  # noqa: F401
