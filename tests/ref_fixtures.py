"""The reference's own test meshes (src/test/test_data/) as committed
fixtures (tests/golden/ref_meshes.npz, made by tests/golden/make_ref_meshes.py),
and the inputs LevelSet::solveLevelSet uses when the caller sets none
(src/LevelSet.cu:187-199, 221-233)."""
import os

import numpy as np

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_meshes.npz")
TETGEN = ("sphere334", "torus", "pyramid")
PLY = ("SquareMesh_size16", "sphere_266verts")


def load(name):
    """(xyz float32 [nv, 3], elements int32 0-based in file order, index base)."""
    with np.load(FIXTURE) as z:
        return z[name + "_xyz"], z[name + "_elems"], int(z[name + "_first"])


def sha256(name):
    with np.load(FIXTURE) as z:
        return str(z[name + "_sha256"])


def reference_data_dir():
    """The reference's test_data directory when LS_REFERENCE_ROOT names a
    reference tree, else None (tests that read the original files skip)."""
    root = os.environ.get("LS_REFERENCE_ROOT", "")
    d = os.path.join(root, "src", "test", "test_data") if root else ""
    return d if d and os.path.isdir(d) else None


def default_inputs(dim, xyz, ne):
    """phi0 = x - midX; velocity (rangeX / 100, 0, 0) per element in 3D and
    zero in 2D, as the reference's solveLevelSet sets them."""
    x = np.asarray(xyz, np.float32)[:, 0].astype(np.float64)
    lo, hi = float(x.min()), float(x.max())
    phi0 = (x - (lo + hi) / 2.0).astype(np.float32)
    vel = np.zeros((ne, 3), np.float32)
    if dim == 3:
        vel[:, 0] = np.float32((hi - lo) / 100.0)
    return phi0, vel
