"""Mesh readers and the VTK writer behind ls_load_mesh / ls_write_vtk
(the file formats LevelSet::initializeMesh loads, src/LevelSet.cu:111-144,
and meshFIM3d::writeVTK writes, src/core3d/cuda/meshFIM3d.cu:48-81)."""
import os

import numpy as np
import pytest

import lsgb300
import lsoracle
import ref_fixtures
import synth


def _parse_tetgen(base):
    def rows(path):
        out = []
        for line in open(path):
            line = line.split("#")[0].split()
            if line:
                out.append(line)
        return out

    nodes, eles = rows(base + ".node"), rows(base + ".ele")
    nn, ne = int(nodes[0][0]), int(eles[0][0])
    first = int(nodes[1][0])
    xyz = np.array([[float(v) for v in r[1:4]] for r in nodes[1:nn + 1]], np.float32)
    tets = np.array([[int(v) - first for v in r[1:5]] for r in eles[1:ne + 1]], np.int32)
    return xyz, tets


def _parse_ply(path):
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


@pytest.mark.parametrize("first", [0, 1])
def test_tetgen_roundtrip(tmp_path, first):
    xyz, el = synth.cube_mesh(5, 0.2, seed=3)
    # flip half the tets so that the loader's orientation rule has work
    el = el.copy()
    el[::2, [2, 3]] = el[::2, [3, 2]]
    base = str(tmp_path / "cube")
    synth.write_tetgen(base, xyz, el, first=first)
    for name in (base, base + ".node", base + ".ele"):
        ls = lsgb300.LevelSet(False)
        x, t = ls.load_mesh(name)
        assert np.array_equal(x, np.asarray(xyz, np.float32))
        assert np.array_equal(t, synth.reorient(xyz, el))


def test_ply_roundtrip_with_quads(tmp_path):
    n = 6
    g = np.stack(np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="xy"), -1).reshape(-1, 2)
    xyz = np.concatenate([g * 0.25, np.zeros((len(g), 1))], 1)
    faces = []
    for j in range(n):
        for i in range(n):
            a = j * (n + 1) + i
            faces.append((a, a + 1, a + n + 2, a + n + 1))  # quads: split into two triangles
    faces.append((0, 1, n + 1))
    path = str(tmp_path / "sq.ply")
    synth.write_ply(path, xyz, faces)
    ls = lsgb300.LevelSet(True)
    x, t = ls.load_mesh(path)
    ex, et = _parse_ply(path)
    assert np.array_equal(x, ex) and np.array_equal(t, et)
    assert len(t) == 2 * n * n + 1


def test_ply_one_based(tmp_path):
    xyz = [[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]]
    path = str(tmp_path / "one.ply")
    synth.write_ply(path, xyz, [(1, 2, 3), (2, 4, 3)])
    _, t = lsgb300.LevelSet(True).load_mesh(path)
    assert np.array_equal(t, [[0, 1, 2], [1, 3, 2]])


def test_vtk_writer(tmp_path):
    xyz, el = synth.cube_mesh(3, 0.1, seed=1)
    ls = lsgb300.LevelSet(False)
    ls.set_mesh(xyz, el)
    phi = np.linspace(-1, 1, len(xyz)).astype(np.float32)
    path = str(tmp_path / "out.vtk")
    ls.write_vtk(path, phi)
    lines = open(path).read().splitlines()
    assert lines[0].startswith("# vtk DataFile") and lines[3] == "DATASET UNSTRUCTURED_GRID"
    nv = int(lines[4].split()[1])
    pts = np.array([[float(v) for v in lines[5 + i].split()] for i in range(nv)], np.float32)
    assert np.array_equal(pts, np.asarray(xyz, np.float32))
    k = 5 + nv
    ne, tot = map(int, lines[k].split()[1:])
    assert ne == len(el) and tot == 5 * ne
    cells = np.array([[int(v) for v in lines[k + 1 + e].split()] for e in range(ne)])
    assert np.all(cells[:, 0] == 4) and np.array_equal(cells[:, 1:], el)
    k += 1 + ne
    assert lines[k] == "CELL_TYPES %d" % ne and all(lines[k + 1 + e] == "10" for e in range(ne))
    k += 1 + ne
    assert lines[k] == "POINT_DATA %d" % nv and lines[k + 1].startswith("SCALARS traveltime float")
    vals = np.array([float(lines[k + 3 + i]) for i in range(nv)], np.float32)
    assert np.array_equal(vals, phi)


def test_bad_files(tmp_path):
    ls = lsgb300.LevelSet(False)
    with pytest.raises(lsgb300.LevelSetError) as e:
        ls.load_mesh(str(tmp_path / "missing"))
    assert e.value.code == lsgb300.LS_BAD_INPUT
    base = str(tmp_path / "bad")
    with open(base + ".node", "w") as f:
        f.write("4 3 0 0\n0 0 0 0\n1 1 0 0\n")  # truncated
    with open(base + ".ele", "w") as f:
        f.write("1 4 0\n0 0 1 2 3\n")
    with pytest.raises(lsgb300.LevelSetError):
        ls.load_mesh(base)
    with open(base + ".node", "w") as f:
        f.write("4 3 0 0\n0 0 0 0\n1 1 0 0\n2 0 1 0\n3 0 0 1\n")
    with open(base + ".ele", "w") as f:
        f.write("1 4 0\n0 0 1 2 9\n")  # vertex out of range
    with pytest.raises(lsgb300.LevelSetError):
        ls.load_mesh(base)
    p = str(tmp_path / "oob.ply")
    synth.write_ply(p, [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [(0, 1, 3)])
    with pytest.raises(lsgb300.LevelSetError):
        lsgb300.LevelSet(True).load_mesh(p)
    p = str(tmp_path / "bin.ply")
    with open(p, "w") as f:
        f.write("ply\nformat binary_little_endian 1.0\nelement vertex 3\nend_header\n")
    with pytest.raises(lsgb300.LevelSetError):
        lsgb300.LevelSet(True).load_mesh(p)


def _ref_file(name):
    d = ref_fixtures.reference_data_dir()
    if d is None or not os.path.exists(os.path.join(d, name)):
        pytest.skip("reference tree not given (LS_REFERENCE_ROOT)")
    return os.path.join(d, name)


@pytest.mark.parametrize("name", ref_fixtures.TETGEN)
def test_reference_tetgen_fixtures(name):
    """The original files, where the reference tree is given: the loader's
    result equals the committed fixture (reoriented)."""
    base = _ref_file(name + ".node")[:-5]
    ls = lsgb300.LevelSet(False)
    x, t = ls.load_mesh(base)
    ex, et = _parse_tetgen(base)
    fx, fe, _ = ref_fixtures.load(name)
    assert np.array_equal(ex, fx) and np.array_equal(et, fe)
    assert np.array_equal(x, ex)
    assert np.array_equal(t, synth.reorient(ex, et))


@pytest.mark.parametrize("name", ref_fixtures.PLY + ("sphere_1154verts",))
def test_reference_ply_fixtures(name):
    path = _ref_file(name + ".ply")
    ls = lsgb300.LevelSet(True)
    x, t = ls.load_mesh(path)
    ex, et = _parse_ply(path)
    assert np.array_equal(x, ex) and np.array_equal(t, et)
    if name in ref_fixtures.PLY:
        fx, fe, _ = ref_fixtures.load(name)
        assert np.array_equal(ex, fx) and np.array_equal(et, fe)


@pytest.mark.parametrize("name", ref_fixtures.TETGEN + ref_fixtures.PLY)
def test_fixture_meshes_through_loader(tmp_path, name):
    """The reference's meshes (committed fixtures), written back in their
    file format with the file's index base, load to the same arrays; tetgen
    meshes come back with the loader's orientation fix-up applied."""
    xyz, el, first = ref_fixtures.load(name)
    if name in ref_fixtures.TETGEN:
        base = str(tmp_path / name)
        synth.write_tetgen(base, xyz, el, first=first)
        x, t = lsgb300.LevelSet(False).load_mesh(base)
        assert np.array_equal(t, synth.reorient(xyz, el))
    else:
        path = str(tmp_path / (name + ".ply"))
        synth.write_ply(path, xyz, [tuple(r) for r in el])
        x, t = lsgb300.LevelSet(True).load_mesh(path)
        assert np.array_equal(t, el)
    assert np.array_equal(x, xyz)


def test_reference_fixture_layout_matches_oracle():
    """The reference's sphere334 mesh (committed fixture), oriented as the
    loader leaves it and RCB-partitioned, gives the same patch layout as the
    restatement of the reference's layout code."""
    xyz, el, _ = ref_fixtures.load("sphere334")
    t = synth.reorient(xyz, el)
    ls = lsgb300.LevelSet(False)
    ls.set_mesh(xyz, t)
    npart, nparts = lsgb300.partition_rcb(3, xyz, 16)
    ls.set_partition(npart, nparts)
    ls.prepare()
    ol = lsoracle.OracleLayout(3, xyz, t, npart, nparts)
    for a in lsgb300.REF_ARRAYS:
        assert np.array_equal(ls.layout(a), ol.array(a)), a
