"""Loading helpers for the committed golden fixtures (tests/golden/*.npz)."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name: str):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def names(prefix: str):
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))
