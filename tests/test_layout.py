"""Patch layout: the product's host layout builder reproduces the reference's
layout arrays (oracle restatement of meshFIM3d.cu:423-570) bit for bit."""
import numpy as np
import pytest

import lsgb300
import lsoracle
import ref_fixtures
import synth

ARRAYS = list(lsgb300.REF_ARRAYS)


def _compare(dim, xyz, el, npart, nparts):
    ls = lsgb300.LevelSet(dim == 2)
    ls.set_mesh(xyz, el)
    ls.set_partition(npart, nparts)
    ls.prepare()
    ol = lsoracle.OracleLayout(dim, xyz, el, npart, nparts)
    info = ls.layout_info()
    for k in ("nparts", "full", "lep", "lvp", "lim", "nadj", "nv", "ne"):
        assert info[k] == ol.info[k], k
    for a in ARRAYS:
        x, y = ls.layout(a), ol.array(a)
        assert x.dtype == y.dtype and x.shape == y.shape, a
        assert np.array_equal(x, y), a
    return ls, ol


@pytest.mark.parametrize("n,block", [(6, 3), (8, 3), (9, 4), (7, 2)])
def test_layout_cube_structured(n, block):
    xyz, el = synth.cube_mesh(n, 0.15, seed=n)
    npart, nparts = synth.structured_partition(3, n + 1, block)
    _compare(3, xyz, el, npart, nparts)


@pytest.mark.parametrize("n,block", [(16, 5), (20, 4), (11, 3)])
def test_layout_square_structured(n, block):
    xyz, el = synth.square_mesh(n, 0.2, seed=n)
    npart, nparts = synth.structured_partition(2, n + 1, block)
    _compare(2, xyz, el, npart, nparts)


def test_layout_graph_partition():
    xyz, el = synth.cube_mesh(7, 0.15, seed=1)
    npart, nparts = lsgb300.partition_rcb(3, xyz, 20)
    assert nparts == int(np.ceil(len(xyz) / 20))
    _compare(3, xyz, el, npart, nparts)


def test_layout_shuffled_elements():
    # element order and vertex order inside elements drive the copy order
    rng = np.random.default_rng(5)
    xyz, el = synth.cube_mesh(6, 0.1, seed=2)
    el = el[rng.permutation(len(el))]
    el = np.take_along_axis(el, np.argsort(rng.random(el.shape), 1), 1)
    npart, nparts = synth.structured_partition(3, 7, 3)
    _compare(3, xyz, el, npart, nparts)


def test_structured_partition_matches_reference_labels():
    for dim, side, b in [(3, 9, 3), (3, 10, 4), (2, 13, 5)]:
        nv = side ** dim
        a, na = lsgb300.partition_structured(dim, side, b, nv)
        c, nc = synth.structured_partition(dim, side, b)
        assert na == nc and np.array_equal(a, c)


def test_cube_numbering_matches_reference_fixture():
    # CubeMesh_size256step8_correct.node lists 33^3 vertices, x fastest,
    # spacing 8: vertex 1 = (8,0,0), vertex 33 = (0,8,0), vertex 33^2 = (0,0,8)
    xyz, _ = synth.cube_mesh(32, 0.0, scale=256.0)
    assert len(xyz) == 35937
    np.testing.assert_allclose(xyz[1], [8, 0, 0])
    np.testing.assert_allclose(xyz[33], [0, 8, 0])
    np.testing.assert_allclose(xyz[33 * 33], [0, 0, 8])
    np.testing.assert_allclose(xyz[-1], [256, 256, 256])


def test_bad_inputs_return_status():
    ls = lsgb300.LevelSet(False)
    with pytest.raises(lsgb300.LevelSetError) as e:
        ls.set_phi(np.zeros(3, np.float32))
    assert e.value.code == lsgb300.LS_BAD_INPUT
    xyz, el = synth.cube_mesh(3, 0.0)
    bad = el.copy()
    bad[0, 0] = 10 ** 6
    with pytest.raises(lsgb300.LevelSetError):
        ls.set_mesh(xyz, bad)
    ls.set_mesh(xyz, el)
    with pytest.raises(lsgb300.LevelSetError):
        ls.set_partition(np.full(len(xyz), 7, np.int32), 3)
    # a patch without vertices is rejected at preparation
    npart = np.zeros(len(xyz), np.int32)
    ls.set_partition(npart, 2)
    with pytest.raises(lsgb300.LevelSetError):
        ls.prepare()
    with pytest.raises(lsgb300.LevelSetError) as e:
        ls.solve(1)
    assert e.value.code == lsgb300.LS_NOT_READY


def test_patch_too_large_is_reported():
    xyz, el = synth.cube_mesh(8, 0.0)
    ls = lsgb300.LevelSet(False)
    ls.set_mesh(xyz, el)
    ls.set_partition(np.zeros(len(xyz), np.int32), 1)
    with pytest.raises(lsgb300.LevelSetError) as e:
        ls.prepare()
    assert e.value.code == lsgb300.LS_PATCH_TOO_LARGE


@pytest.mark.parametrize("name,target", [("sphere334", 16), ("torus", 16), ("pyramid", 3)])
def test_reference_fixture_meshes(name, target):
    """The reference's own tetgen meshes (committed fixtures), RCB-partitioned."""
    xyz, el, _ = ref_fixtures.load(name)
    npart, nparts = lsgb300.partition_rcb(3, xyz, target)
    _compare(3, xyz, el, npart, nparts)
