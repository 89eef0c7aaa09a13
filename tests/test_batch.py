"""Batches of independent meshes (ls_batch_*): the merged patch layout is the
layout of the disjoint union (CPU), and on the GPU every member of a batch
steps exactly as it does alone (bit for bit), each with its own time step,
bandwidth and FIM length unit."""
import numpy as np
import pytest

import lsgb300
import synth


def _member(w, **kw):
    return lsgb300.from_workload(w, setup=False, **kw)


def _small_batch(dim=3):
    if dim == 3:
        ws = [synth.workload("c2", n=6), synth.workload("c3", n=9), synth.workload("c2", n=8, seed=3)]
        # one advection kind for the whole batch
        ws[1] = dict(ws[1], update="advect", vel=synth.velocity_rotation(ws[1]["xyz"], ws[1]["elems"], 3.0))
    else:
        ws = [synth.workload("c1", n=12), synth.workload("c1", n=20, seed=2), synth.workload("c1", n=16, seed=5)]
    return ws


@pytest.mark.parametrize("dim", [2, 3])
def test_merged_layout_is_union_layout(dim):
    ws = _small_batch(dim)
    b = lsgb300.LevelSetBatch()
    for w in ws:
        b.add(_member(w))
    xyz = np.concatenate([w["xyz"] for w in ws])
    el, npart, vb, pb = [], [], 0, 0
    for w in ws:
        el.append(w["elems"] + vb)
        npart.append(w["npart"] + pb)
        vb += len(w["xyz"])
        pb += w["nparts"]
    u = lsgb300.LevelSet(dim == 2)
    u.set_mesh(xyz, np.concatenate(el))
    u.set_partition(np.concatenate(npart), pb)
    u.prepare()
    bi, ui = b.layout_info(), u.layout_info()
    for k in ("nparts", "full", "lep", "lvp", "lgp", "lim", "nadj", "nv", "ne", "dim"):
        assert bi[k] == ui[k], k
    for name in lsgb300.REF_ARRAYS:
        assert np.array_equal(b.layout(name), u.layout(name)), name


def test_batch_rejects_mixed_members():
    b = lsgb300.LevelSetBatch()
    b.add(_member(synth.workload("c2", n=6)))
    with pytest.raises(lsgb300.LevelSetError):
        b.add(_member(synth.workload("c1", n=8)))  # 2D into a 3D batch
    with pytest.raises(lsgb300.LevelSetError):
        b.add(_member(dict(synth.workload("c2", n=6), update="curvature")))
    with pytest.raises(lsgb300.LevelSetError):
        lsgb300.LevelSetBatch().setup()  # empty


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("bit_exact", [True, False])
def test_batch_members_step_as_alone(dim, bit_exact):
    ws = _small_batch(dim)
    nsteps = 4
    b = lsgb300.LevelSetBatch()
    alone = []
    for w in ws:
        b.add(_member(w, bit_exact=bit_exact))
        ls = lsgb300.from_workload(w, bit_exact=bit_exact)
        hist, done = ls.solve(nsteps)
        assert done == nsteps
        alone.append((hist[-1], ls.stats()))
    b.setup()
    assert b.solve(nsteps) == nsteps
    st = b.stats()
    for i, (ref, _) in enumerate(alone):
        assert np.array_equal(b.phi(i).view(np.uint32), ref.view(np.uint32)), i
    for k in ("patch_visits", "check_visits", "nb_vertex_updates", "nb_patches"):
        assert st[k] == sum(s[k] for _, s in alone), k
    # FIM iterations of a batch step: the slowest member's
    assert st["fim_iters"] <= sum(s["fim_iters"] for _, s in alone)


@pytest.mark.gpu
def test_batch_curvature_members_and_profile_path():
    ws = [synth.workload("c3", n=10), synth.workload("c3", n=14, seed=1)]
    b = lsgb300.LevelSetBatch()
    refs = []
    for w in ws:
        b.add(_member(w, bit_exact=True))
        ls = lsgb300.from_workload(w, bit_exact=True)
        hist, _ = ls.solve(3)
        refs.append(hist[-1])
    b.setup()
    b.set_profile(True)  # launch-by-launch path
    b.solve(3)
    for i, ref in enumerate(refs):
        assert np.array_equal(b.phi(i).view(np.uint32), ref.view(np.uint32)), i


@pytest.mark.gpu
def test_batch_autotune_leaves_best_setting():
    # patch side and FIM setting tuned over the merged batch; the batch is
    # left set up with the best at phi0 and steps as a batch built directly
    # with those settings
    ws = synth.workload_batch(seed=3, nmesh=4, nmin=8, nmax=16)

    def batch(block, ctas=None):
        b = lsgb300.LevelSetBatch()
        for w in ws:
            extra = {"fim_ctas_per_sm": ctas} if ctas else {}
            b.add(lsgb300.from_workload(w, setup=False, structured_block=block, **extra))
        return b

    b = batch(3)
    trials, best = b.autotune(1)
    assert {t["patch_size"] for t in trials} == {2, 3, 4}
    assert trials[best]["updates_per_s"] == max(t["updates_per_s"] for t in trials)
    b.solve(3)
    c = batch(trials[best]["patch_size"], trials[best]["fim_ctas_per_sm"])
    c.setup()
    c.solve(3)
    for i in range(len(ws)):
        assert np.array_equal(b.phi(i).view(np.uint32), c.phi(i).view(np.uint32)), i
