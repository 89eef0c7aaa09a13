"""GPU: the persistent FIM loop (LS_PERSISTENT) -- every FIM iteration of a
step in one cooperative launch, the sweep, schedule and check passes
separated by grid-wide barriers -- against the launch-per-pass step: same
bits, same work counters; the bit-exact build's persistent step against the
oracle; batches; the graph and kernel-by-kernel forms; and a grid-barrier
wait that runs out (limit of one poll) ending the step with
LS_DEVICE_TIMEOUT while the handle and the GPU stay usable."""
import numpy as np
import pytest

import lsgb300
import lsoracle
import synth

pytestmark = pytest.mark.gpu

KEYS = ("fim_iters", "patch_visits", "check_visits", "nb_vertex_updates", "nb_patches", "early_visits")


def _run(w, nsteps, **kw):
    ls = lsgb300.from_workload(w, **kw)
    hist, done = ls.solve(nsteps)
    return hist, done, ls.stats()


@pytest.mark.parametrize("name,n,update", [("c3", 24, None), ("c2", 12, None), ("c3", 96, "curvature")])
def test_fast_build_persistent_equals_launch_per_pass(name, n, update):
    w = synth.workload(name, n=n)
    if update:
        w["update"] = update
    nsteps = 3
    h0, d0, s0 = _run(w, nsteps)
    h1, d1, s1 = _run(w, nsteps, flags=lsgb300.PERSISTENT)
    assert d0 == d1 == nsteps
    assert np.array_equal(h0.view(np.uint32), h1.view(np.uint32))
    for k in KEYS:
        assert s0[k] == s1[k], k


@pytest.mark.parametrize("name,n", [("c1", 16), ("c2", 9), ("c3", 14)])
@pytest.mark.parametrize("ref_compat", [False, True])
def test_bitexact_persistent_equals_oracle(name, n, ref_compat):
    w = synth.workload(name, n=n)
    nsteps = 4
    ls = lsgb300.from_workload(w, bit_exact=True, ref_compat=ref_compat, flags=lsgb300.PERSISTENT)
    hist, done = ls.solve(nsteps)
    ol = lsoracle.OracleLayout(w["dim"], w["xyz"], w["elems"], w["npart"], w["nparts"])
    p = ol.params(update_kind=lsoracle.UPDATE[w["update"]], dt=w["dt"], bandwidth=w["bandwidth"], curv_coeff=1.0,
                  ref_compat=1 if ref_compat else 0)
    ref, nbs, _, ost = ol.solve(p, w["phi0"], w["vel"], nsteps)
    assert done == ost["steps_run"] == nsteps
    assert np.array_equal(hist.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(ls.narrowband(w["nparts"]), nbs[-1])
    st = ls.stats()
    for k in ("fim_iters", "patch_visits", "check_visits", "nb_vertex_updates"):
        assert st[k] == ost[k], k


@pytest.mark.parametrize("flags", [lsgb300.NO_GRAPH, lsgb300.PROFILE])
def test_persistent_kernel_by_kernel_equals_graph(flags):
    w = synth.workload("c3", n=20)
    h0, _, s0 = _run(w, 3, flags=lsgb300.PERSISTENT)
    h1, _, s1 = _run(w, 3, flags=lsgb300.PERSISTENT | flags)
    assert np.array_equal(h0.view(np.uint32), h1.view(np.uint32))
    for k in KEYS:
        assert s0[k] == s1[k], k
    if flags == lsgb300.PROFILE:
        assert s1["n_sweep"] == 3 and s1["ms_sweep"] > 0


def test_persistent_batch_equals_launch_per_pass():
    ws = synth.workload_batch(seed=11, nmesh=6, nmin=8, nmax=16)
    out = []
    for flags in (0, lsgb300.PERSISTENT):
        b = lsgb300.LevelSetBatch()
        members = [lsgb300.from_workload(w, setup=False, flags=flags) for w in ws]
        for m in members:
            b.add(m)
        b.setup()
        b.solve(3)
        out.append(([b.phi(i) for i in range(len(ws))], b.stats()))
    for a, c in zip(out[0][0], out[1][0]):
        assert np.array_equal(a.view(np.uint32), c.view(np.uint32))
    for k in ("fim_iters", "patch_visits", "check_visits", "nb_vertex_updates"):
        assert out[0][1][k] == out[1][1][k], k


def test_grid_barrier_wait_runs_out():
    # one poll per barrier wait: the CTAs that reach the first barrier early
    # give up, raise the abort word and leave; the others see it and leave
    # too; the step reports LS_DEVICE_TIMEOUT and the GPU stays usable
    w = synth.workload("c3", n=24)
    ls = lsgb300.from_workload(w, flags=lsgb300.PERSISTENT, barrier_wait_limit=1)
    with pytest.raises(lsgb300.LevelSetError) as e:
        ls.step(1)
    assert e.value.code == lsgb300.LS_DEVICE_TIMEOUT
    # the same handle steps again from phi0 with a normal limit, and matches
    # a fresh handle
    p = ls.get_params()
    p.barrier_wait_limit = 0
    ls.set_params(p)
    ls.setup()
    ls.set_phi(w["phi0"])
    h1, d1 = ls.solve(2)
    h0, d0, _ = _run(w, 2, flags=lsgb300.PERSISTENT)
    assert d0 == d1 == 2
    assert np.array_equal(h0.view(np.uint32), h1.view(np.uint32))
