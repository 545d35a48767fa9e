"""Shared helpers for the tests: fixture loading and the oracle grid."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def golden_names(prefix):
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def seps(f):
    """Separations the reference computed from the fixture's node coordinates."""
    if "ref_hx" in f:
        return f["ref_hx"], f["ref_hy"], f["ref_hz"]
    return tuple(np.diff(f[k]) for k in ("x_nodes", "y_nodes", "z_nodes"))
