"""Partitioners behind partition_type: the graph partitioner (recursive graph
bisection + refinement, the METIS stand-in), recursive coordinate bisection
and GraphPartition_Square blocks."""
import numpy as np
import pytest

import lsgb300
import ref_fixtures
import synth


def _check(npart, nparts, nv, target, dim=3):
    expect = int(np.ceil(nv / target)) if dim == 3 else max(2, nv // target)
    assert nparts == min(expect, nv)
    assert npart.min() == 0 and npart.max() == nparts - 1
    sizes = np.bincount(npart, minlength=nparts)
    assert sizes.min() > 0
    ideal = nv / nparts
    assert sizes.max() <= np.ceil(ideal * 1.03) + 1 + 1


@pytest.mark.parametrize("n,target", [(12, 27), (20, 16), (16, 64)])
def test_graph_partition_cube(n, target):
    xyz, el = synth.cube_mesh(n, 0.15, seed=n)
    nv = len(xyz)
    pg, ng = lsgb300.partition_graph(3, el, nv, target)
    _check(pg, ng, nv, target)
    pr, nr = lsgb300.partition_rcb(3, xyz, target)
    rnd = np.random.default_rng(0).integers(0, ng, nv).astype(np.int32)
    cut_g = lsgb300.edge_cut(3, el, nv, pg)
    assert cut_g < lsgb300.edge_cut(3, el, nv, pr)
    assert cut_g < 0.6 * lsgb300.edge_cut(3, el, nv, rnd)


def test_graph_partition_square_and_shuffled_numbering():
    xyz, el = synth.square_mesh(40, 0.2, seed=3)
    perm = np.random.default_rng(1).permutation(len(xyz)).astype(np.int32)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm), dtype=np.int32)
    el2 = inv[el]  # vertex numbering shuffled: the graph is the same
    pg, ng = lsgb300.partition_graph(2, el2, len(xyz), 25)
    _check(pg, ng, len(xyz), 25, dim=2)
    a = lsgb300.edge_cut(2, el2, len(xyz), pg)
    p0, _ = lsgb300.partition_graph(2, el, len(xyz), 25)
    b = lsgb300.edge_cut(2, el, len(xyz), p0)
    assert a < 1.3 * b and b < 1.3 * a


def test_graph_partition_disconnected_mesh():
    xyz1, el1 = synth.cube_mesh(6, 0.1, seed=1)
    xyz2, el2 = synth.cube_mesh(5, 0.1, seed=2)
    xyz = np.concatenate([xyz1, xyz2 + 3.0]).astype(np.float32)
    el = np.concatenate([el1, el2 + len(xyz1)])
    pg, ng = lsgb300.partition_graph(3, el, len(xyz), 27)
    _check(pg, ng, len(xyz), 27)


def test_graph_partition_bad_input():
    xyz, el = synth.cube_mesh(3, 0.0)
    with pytest.raises(lsgb300.LevelSetError):
        lsgb300.partition_graph(3, el, len(xyz) - 5, 8)  # vertex index out of range
    with pytest.raises(lsgb300.LevelSetError):
        lsgb300.partition_graph(4, el, len(xyz), 8)


def test_handle_partition_types():
    xyz, el = synth.cube_mesh(8, 0.15, seed=4)
    nv = len(xyz)
    for ptype in (0, 2, 1):
        p = lsgb300.default_params(partition_type=ptype, metis_size=27, side_lengths=9, block_size=3)
        ls = lsgb300.LevelSet(False, p)
        ls.set_mesh(xyz, el)
        ls.prepare()
        info = ls.layout_info()
        assert info["nparts"] == (27 if ptype == 1 else int(np.ceil(nv / 27)))


def test_reference_mesh_graph_partition():
    # the reference's torus mesh (committed fixture)
    xyz, el, _ = ref_fixtures.load("torus")
    pg, ng = lsgb300.partition_graph(3, el, len(xyz), 16)
    _check(pg, ng, len(xyz), 16)
    pr, _ = lsgb300.partition_rcb(3, xyz, 16)
    assert lsgb300.edge_cut(3, el, len(xyz), pg) <= 1.1 * lsgb300.edge_cut(3, el, len(xyz), pr)
