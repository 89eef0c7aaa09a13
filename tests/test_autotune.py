"""Autotuner (ls_autotune): picks the patch size and FIM CTAs per SM with the
highest measured throughput and leaves the handle set up with them."""
import numpy as np
import pytest

import lsgb300
import synth


def test_autotune_needs_a_mesh():
    ls = lsgb300.LevelSet(False)
    with pytest.raises(lsgb300.LevelSetError) as e:
        ls.autotune(1)
    assert e.value.code == lsgb300.LS_BAD_INPUT


def _handle(w, **kw):
    p = lsgb300.default_params(time_step=w["dt"], bandwidth=w["bandwidth"], partition_type=1,
                               side_lengths=w["n"] + 1, block_size=3, update_kind=lsgb300.UPDATE_CURVATURE, **kw)
    ls = lsgb300.LevelSet(False, p)
    ls.set_mesh(w["xyz"], w["elems"])
    ls.set_phi(w["phi0"])
    ls.set_velocity(w["vel"])
    return ls


@pytest.mark.gpu
def test_autotune_structured_patches():
    w = synth.workload("c3", n=24)
    ls = _handle(w)
    trials, best = ls.autotune(2)
    sizes = sorted({t["patch_size"] for t in trials})
    assert sizes == [2, 3, 4]
    assert all(t["updates_per_s"] > 0 for t in trials)
    assert trials[best]["updates_per_s"] == max(t["updates_per_s"] for t in trials)
    p = ls.get_params()
    assert p.block_size == trials[best]["patch_size"] and p.fim_ctas_per_sm == trials[best]["fim_ctas_per_sm"]
    # the tuned handle is set up at phi0: its solve equals a fresh handle with the chosen settings
    h1, d1 = ls.solve(3)
    fresh = _handle(w, fim_ctas_per_sm=p.fim_ctas_per_sm)
    q = fresh.get_params()
    q.block_size = p.block_size
    fresh.set_params(q)
    fresh.setup()
    h2, d2 = fresh.solve(3)
    assert d1 == d2 == 3
    assert np.array_equal(h1.view(np.uint32), h2.view(np.uint32))


@pytest.mark.gpu
def test_autotune_keeps_caller_partition():
    w = synth.workload("c2", n=12)
    ls = lsgb300.from_workload(w, setup=False)
    trials, best = ls.autotune(1)
    assert {t["patch_size"] for t in trials} == {0}
    assert {t["fim_ctas_per_sm"] for t in trials} <= {2, 3, 4, 5, 6, 7}
    hist, done = ls.solve(2)
    assert done == 2
