"""Generate tests/golden/ref_steps.npz: the reference's own time steps.

Runs only where the reference tree is present and oracle/_ref has been built
(python oracle/build_ref.py).  For each case the reference's
meshFIM3d::GenerateData (src/core3d/cuda/meshFIM3d.cu:572-690) -- partition,
patch layout, then per step the seed search, sign capture, FIM redistance
with its host-driven active lists (src/core3d/cuda/redistance3d.cu:10-274),
narrowband and advection update (meshFIM3d.cu:83-99) -- compiled from the
reference's source files, with every kernel run on the CPU
(oracle/ref_host_launch.cpp), steps a mesh; the inputs and the phi history it
returns are stored, so that tests anywhere compare the oracle and the
product's bit-exact build with the reference's own solver bit for bit.  The
reference's semantics throughout: absolute SMALLNUM = 1e-5 and LARGENUM =
1e9 (the values its missing dependency would supply), patch-constant
velocity, lengths in the mesh's own units.

    python tests/golden/make_step_golden.py
"""
import ctypes
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref")
sys.path.insert(0, os.path.join(ROOT, "sci-solver_level-set_gb300"))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)
import lsgb300  # noqa: E402
import ref_fixtures  # noqa: E402
import synth  # noqa: E402
from make_layout_golden import vertex_ring  # noqa: E402

P = ctypes.c_void_p


def reference_steps(xyz, el, npart, nparts, side, block, phi0, vel, nsteps, dt, bandwidth):
    lib = ctypes.CDLL(os.path.join(REF, "libref_layout3d.so"))
    xyz = np.ascontiguousarray(xyz, np.float32)
    el = np.ascontiguousarray(el, np.int32)
    off, adj = vertex_ring(len(xyz), el)
    npart = np.ascontiguousarray(npart, np.int32)
    phi0 = np.ascontiguousarray(phi0, np.float32)
    vel = np.ascontiguousarray(vel, np.float32)
    hist = np.zeros((nsteps + 1, len(xyz)), np.float32)
    n = lib.lsref_solve3d(len(xyz), xyz.ctypes.data_as(P), len(el), el.ctypes.data_as(P), off.ctypes.data_as(P),
                          adj.ctypes.data_as(P), npart.ctypes.data_as(P), int(nparts), int(side), int(block),
                          phi0.ctypes.data_as(P), vel.ctypes.data_as(P), int(nsteps), ctypes.c_float(dt),
                          ctypes.c_float(bandwidth), 1, hist.ctypes.data_as(P))
    if n < 0:
        raise RuntimeError("reference time step failed: %d" % n)
    return hist[: n + 1]


def cases():
    """(name, xyz, elems, npart, nparts, side, block, phi0, vel, nsteps, dt, bandwidth)"""
    # 3D advection family, 9^3 cells, 3^3-vertex blocks from the reference's
    # GraphPartition_Square
    w = synth.workload("c2", n=9)
    yield ("c2_9_advect", w["xyz"], w["elems"], w["npart"], w["nparts"], 10, 3, w["phi0"], w["vel"], 4, w["dt"],
           w["bandwidth"])
    # the same mesh, graph-partitioned (the reference's METIS path with these
    # labels), 12^3 cells
    w = synth.workload("c2", n=12)
    npart, nparts = lsgb300.partition_graph(3, w["elems"], len(w["xyz"]), 27)
    yield ("c2_12_graph_advect", w["xyz"], w["elems"], npart, nparts, 0, 0, w["phi0"], w["vel"], 3, w["dt"],
           w["bandwidth"])
    # curvature family's three spheres, redistance only (zero velocity: the
    # reference has no device curvature update)
    w = synth.workload("c3", n=12)
    yield ("c3_12_redistance", w["xyz"], w["elems"], w["npart"], w["nparts"], 13, 3, w["phi0"],
           np.zeros((len(w["elems"]), 3), np.float32), 3, w["dt"], w["bandwidth"])
    # the reference's own meshes with the inputs and parameters its
    # LevelSet::solveLevelSet uses when the caller sets none
    # (src/LevelSet.cu:187-233; time step 1, bandwidth 16, 16-vertex patches)
    p0 = lsgb300.default_params()
    for name in ("sphere334", "torus"):
        xyz, el, _ = ref_fixtures.load(name)
        el = synth.reorient(xyz, el)
        npart, nparts = lsgb300.partition_graph(3, el, len(xyz), 16)
        phi0, vel = ref_fixtures.default_inputs(3, xyz, len(el))
        yield (name + "_defaults", xyz, el, npart, nparts, 0, 0, phi0, vel, 3, p0.time_step, p0.bandwidth)


def main():
    if not os.path.exists(os.path.join(REF, "libref_layout3d.so")):
        print("oracle/_ref not built (python oracle/build_ref.py)")
        return 1
    out = {}
    names = []
    for name, xyz, el, npart, nparts, side, block, phi0, vel, nsteps, dt, bw in cases():
        t = time.time()
        hist = reference_steps(xyz, el, npart, nparts, side, block, phi0, vel, nsteps, dt, bw)
        names.append(name)
        for k, v in (("xyz", np.asarray(xyz, np.float32)), ("elems", np.asarray(el, np.int32)),
                     ("npart", np.asarray(npart, np.int32)), ("nparts", np.int32(nparts)),
                     ("side", np.int32(side)), ("block", np.int32(block)), ("phi0", np.asarray(phi0, np.float32)),
                     ("vel", np.asarray(vel, np.float32)), ("dt", np.float64(dt)), ("bandwidth", np.float64(bw)),
                     ("history", hist)):
            out[name + ":" + k] = v
        print("%s: %d vertices, %d steps, %.1f s" % (name, len(xyz), len(hist) - 1, time.time() - t))
    out["cases"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "ref_steps.npz"), **out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
