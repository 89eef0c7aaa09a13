"""Generate tests/golden/ref_meshes.npz from the reference's own test meshes.

Reads the tetgen (.node/.ele) and ASCII PLY meshes the reference ships in
src/test/test_data/ (the inputs LevelSet::initializeMesh loads,
src/LevelSet.cu:111-144) with the small text parsers below, and stores the
parsed arrays so that tests on machines without the reference tree (the GPU
box included) can run the same meshes through the loader, the layout and
the time step:

  <name>_xyz     float32 [nv, 3]   vertex coordinates as written in the file
  <name>_elems   int32 [ne, 4|3]   elements, 0-based, in file order and
                                   orientation (PLY polygons fanned)
  <name>_first   int32             index base of the file (tetgen)
  <name>_sha256  str               digest of the source file(s)

    python tests/golden/make_ref_meshes.py [REFERENCE_ROOT]

REFERENCE_ROOT defaults to the LS_REFERENCE_ROOT environment variable.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TETGEN = ["sphere334", "torus", "pyramid"]
PLY = ["SquareMesh_size16", "sphere_266verts"]


def _rows(path):
    out = []
    for line in open(path):
        line = line.split("#")[0].split()
        if line:
            out.append(line)
    return out


def parse_tetgen(base):
    nodes, eles = _rows(base + ".node"), _rows(base + ".ele")
    nn, ne = int(nodes[0][0]), int(eles[0][0])
    first = int(nodes[1][0])
    xyz = np.array([[float(v) for v in r[1:4]] for r in nodes[1:nn + 1]], np.float32)
    tets = np.array([[int(v) - first for v in r[1:5]] for r in eles[1:ne + 1]], np.int32)
    return xyz, tets, first


def parse_ply(path):
    lines = open(path).read().splitlines()
    nv = nf = 0
    i = 0
    while lines[i].strip() != "end_header":
        w = lines[i].split()
        if w[:2] == ["element", "vertex"]:
            nv = int(w[2])
        if w[:2] == ["element", "face"]:
            nf = int(w[2])
        i += 1
    i += 1
    xyz = np.array([[float(v) for v in lines[i + k].split()[:3]] for k in range(nv)], np.float32)
    tris = []
    for k in range(nf):
        w = [int(v) for v in lines[i + nv + k].split()]
        for j in range(1, w[0] - 1):
            tris.append((w[1], w[1 + j], w[2 + j]))
    tris = np.array(tris, np.int32)
    if tris.min() == 1 and tris.max() == nv:  # 1-based file
        tris -= 1
    return xyz, tris


def _digest(paths):
    h = hashlib.sha256()
    for p in paths:
        h.update(open(p, "rb").read())
    return h.hexdigest()


def main(ref_root):
    data = os.path.join(ref_root, "src", "test", "test_data")
    if not os.path.isdir(data):
        print("reference test data not found under", ref_root)
        return 1
    out = {}
    for name in TETGEN:
        base = os.path.join(data, name)
        xyz, tets, first = parse_tetgen(base)
        out[name + "_xyz"], out[name + "_elems"] = xyz, tets
        out[name + "_first"] = np.int32(first)
        out[name + "_sha256"] = np.array(_digest([base + ".node", base + ".ele"]))
    for name in PLY:
        path = os.path.join(data, name + ".ply")
        xyz, tris = parse_ply(path)
        out[name + "_xyz"], out[name + "_elems"] = xyz, tris
        out[name + "_first"] = np.int32(0)
        out[name + "_sha256"] = np.array(_digest([path]))
    np.savez_compressed(os.path.join(HERE, "ref_meshes.npz"), **out)
    for name in TETGEN + PLY:
        print(name, out[name + "_xyz"].shape, out[name + "_elems"].shape)
    return 0


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LS_REFERENCE_ROOT", "")
    sys.exit(main(root) if root else (print("give REFERENCE_ROOT or set LS_REFERENCE_ROOT") or 1))
