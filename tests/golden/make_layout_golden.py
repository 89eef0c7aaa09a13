"""Generate tests/golden/ref_layout.npz: the reference's own patch layout.

Runs only where the reference tree is present and oracle/_ref has been built
(python oracle/build_ref.py).  For each case the reference's meshFIM3d /
meshFIM2d InitPatches, InitPatches2 and GenerateBlockNeighbors
(src/core3d/cuda/meshFIM3d.cu:423-570, src/core2d/cuda/meshFIM2d.cu:447-606),
compiled from the reference's source files with their layout kernels run on
the CPU (oracle/ref_host_launch.cpp), build the layout of a mesh.  Stored per
case: the inputs, and for each of the eleven layout arrays its length and
SHA-256 digest (the arrays themselves as well when the mesh has at most 2,500
element copies), so that tests anywhere compare the product's layout builder
(and the oracle's restatement) with the reference's bit for bit.  Cases with
a "square" partition take the vertex labels from the reference's
GraphPartition_Square (meshFIM3d.cu:269-352, meshFIM2d.cu:299-371) instead
of a given partition.

    python tests/golden/make_layout_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref")
sys.path.insert(0, os.path.join(ROOT, "sci-solver_level-set_gb300"))
sys.path.insert(0, os.path.dirname(HERE))
import lsgb300  # noqa: E402
import ref_fixtures  # noqa: E402
import synth  # noqa: E402

ARRAYS = dict(lsgb300.REF_ARRAYS)
P = ctypes.c_void_p


def vertex_ring(nv, el):
    """Vertex 1-ring as CSR (sorted neighbours), the TetMesh / TriMesh
    neighbour lists the reference's partition functions read."""
    d1 = el.shape[1]
    a = np.repeat(el[:, :, None], d1, 2).reshape(len(el), -1)
    b = np.repeat(el[:, None, :], d1, 1).reshape(len(el), -1)
    m = a != b
    pairs = np.unique(np.stack([a[m], b[m]], 1), axis=0)
    off = np.zeros(nv + 1, np.int64)
    np.add.at(off, pairs[:, 0] + 1, 1)
    return np.cumsum(off).astype(np.int32), np.ascontiguousarray(pairs[:, 1], np.int32)


def reference_layout(dim, xyz, el, npart=None, nparts=0, side=0, block=0):
    lib = ctypes.CDLL(os.path.join(REF, "libref_layout%dd.so" % dim))
    tag = "lsref_layout%dd" % dim
    getattr(lib, tag + "_array").restype = ctypes.c_longlong
    xyz = np.ascontiguousarray(xyz, np.float32)
    el = np.ascontiguousarray(el, np.int32)
    off, adj = vertex_ring(len(xyz), el)
    npp = np.ascontiguousarray(npart, np.int32) if npart is not None else None
    rc = getattr(lib, tag)(len(xyz), xyz.ctypes.data_as(P), len(el), el.ctypes.data_as(P), off.ctypes.data_as(P),
                           adj.ctypes.data_as(P), npp.ctypes.data_as(P) if npp is not None else None, int(nparts),
                           int(side), int(block))
    if rc != 0:
        raise RuntimeError("reference layout failed: %d" % rc)
    info = (ctypes.c_longlong * 7)()
    getattr(lib, tag + "_info")(info)
    out = {"nparts": int(info[2]), "full": int(info[3]), "lep": int(info[4]), "launches": int(info[5])}
    get = getattr(lib, tag + "_array")
    for name, sel in list(ARRAYS.items()) + [("npart", 11)]:
        n = get(sel, None)
        dt = (np.float32 if dim == 3 else np.float64) if name == "local_coords" else np.int32
        a = np.zeros(n, dt)
        get(sel, a.ctypes.data_as(P))
        out[name] = a
    return out


def digest(a):
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def cases():
    w = synth.workload("c2", n=9)
    yield "c2_9", 3, w["xyz"], w["elems"], w["npart"], w["nparts"], 0, 0
    yield "c2_9_square", 3, w["xyz"], w["elems"], None, 0, 10, 3
    w = synth.workload("c1", n=16)
    yield "c1_16", 2, w["xyz"], w["elems"], w["npart"], w["nparts"], 0, 0
    yield "c1_16_square", 2, w["xyz"], w["elems"], None, 0, 17, 5
    for name, target in (("sphere334", 16), ("torus", 16), ("pyramid", 3)):
        xyz, el, _ = ref_fixtures.load(name)
        el = synth.reorient(xyz, el)
        npart, nparts = lsgb300.partition_graph(3, el, len(xyz), target)
        yield name, 3, xyz, el, npart, nparts, 0, 0
    for name in ref_fixtures.PLY:
        xyz, el, _ = ref_fixtures.load(name)
        npart, nparts = lsgb300.partition_graph(2, el, len(xyz), 16)
        yield name, 2, xyz, el, npart, nparts, 0, 0


def main():
    if not os.path.exists(os.path.join(REF, "libref_layout3d.so")):
        print("oracle/_ref not built (python oracle/build_ref.py)")
        return 1
    out = {}
    names = []
    for name, dim, xyz, el, npart, nparts, side, block in cases():
        r = reference_layout(dim, xyz, el, npart, nparts, side, block)
        names.append(name)
        out[name + ":dim"] = np.int32(dim)
        out[name + ":xyz"] = np.ascontiguousarray(xyz, np.float32)
        out[name + ":elems"] = np.ascontiguousarray(el, np.int32)
        out[name + ":side"] = np.int32(side)
        out[name + ":block"] = np.int32(block)
        for k, v in r.items():
            v = np.asarray(v)
            if v.ndim == 0:
                out[name + ":" + k] = v
                continue
            out[name + ":" + k + ":sha256"] = np.array(digest(v))
            out[name + ":" + k + ":len"] = np.int64(v.size)
            if r["full"] <= 2500 or k == "npart":
                out[name + ":" + k] = v
        print(name, "dim", dim, "nparts", r["nparts"], "full", r["full"], "launches", r["launches"])
    out["cases"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "ref_layout.npz"), **out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
