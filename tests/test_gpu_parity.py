"""GPU parity: the sm_103a path through the C ABI against the CPU oracle on
the same seeded inputs (small members of the benchmark families).

Two kernel builds are checked:
  * bit-exact build (LS_BITEXACT: compiled without FMA contraction, every
    float operation in the reference's order): phi history, narrowband sets
    and work counters identical to the oracle, bit for bit, for 2D and 3D,
    advection / curvature / redistance only, with and without the
    reference's semantics and with the precision form;
  * fast build (FMA contraction): >= 98% of the band vertices within 1e-3 h
    of the oracle per step.  The FIM stops a patch when one sweep changes
    it by less than SMALLNUM (1e-5 h in the FIM frame), so two evaluations
    that round differently stop at slightly different points, ~1e-4 h apart
    on many vertices; and two correct FP32 evaluations of the reference
    algorithm that round differently (the oracle compiled with and without
    FMA shows the same spread) differ by up to ~1e-2 h at a few vertices:
    the N-scheme weights of the advection update are 0/0 where the
    velocity is tangent to the level sets, the curvature update divides by
    |grad phi| per element, and the tet solver's face discriminants cancel
    when two arrival times are nearly equal.
"""
import numpy as np
import pytest

import lsgb300
import lsoracle
import synth

pytestmark = pytest.mark.gpu

CASES = [("c1", 16), ("c2", 9), ("c3", 14)]


def _oracle(w, ref_compat, tau, nsteps, precision=32, update=None):
    ol = lsoracle.OracleLayout(w["dim"], w["xyz"], w["elems"], w["npart"], w["nparts"])
    p = ol.params(update_kind=lsoracle.UPDATE[update or w["update"]], dt=w["dt"], bandwidth=w["bandwidth"],
                  curv_coeff=1.0, ref_compat=1 if ref_compat else 0, fp64_tau=tau, precision=precision)
    return ol.solve(p, w["phi0"], w["vel"], nsteps)


def _band_err(a, b, w):
    band = (np.abs(b) <= w["bandwidth"]) & (np.abs(a) <= w["bandwidth"])
    return np.abs(a[band] - b[band]) / w["h"], band


@pytest.mark.parametrize("name,n", CASES)
@pytest.mark.parametrize("ref_compat", [False, True])
@pytest.mark.parametrize("fp64", [False, True])
def test_bitexact_build_equals_oracle(name, n, ref_compat, fp64):
    w = synth.workload(name, n=n)
    nsteps = 4
    tau = 2.0 ** -18 if (fp64 and w["dim"] == 3) else 0.0
    ls = lsgb300.from_workload(w, ref_compat=ref_compat, fp64_flagged=fp64, bit_exact=True)
    hist, done = ls.solve(nsteps)
    st = ls.stats()
    ref, nbs, iters, ost = _oracle(w, ref_compat, tau, nsteps)
    assert done == ost["steps_run"] == nsteps
    assert np.array_equal(hist.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(ls.narrowband(w["nparts"]), nbs[-1])
    for k in ("fim_iters", "patch_visits", "check_visits", "nb_vertex_updates", "nb_patches", "nb_patch_vertices"):
        assert st[k] == ost[k], k


@pytest.mark.parametrize("name,n", CASES)
@pytest.mark.parametrize("ref_compat", [False, True])
@pytest.mark.parametrize("ctas", [3, 6, 7])
def test_bitexact_build_other_sweep_settings_equal_oracle(name, n, ref_compat, ctas):
    # the default setting (5) runs tetrahedra on the two-copies sweep with the
    # reference's solver; 3 keeps the one-copy kernel that runs every solve,
    # 6 the two-copies kernel at six CTAs per SM, 7 the same kernel with one
    # copy per thread: all equal the oracle
    w = synth.workload(name, n=n)
    nsteps = 4
    ls = lsgb300.from_workload(w, ref_compat=ref_compat, bit_exact=True, fim_ctas_per_sm=ctas)
    hist, done = ls.solve(nsteps)
    st = ls.stats()
    ref, nbs, iters, ost = _oracle(w, ref_compat, 0.0, nsteps)
    assert done == ost["steps_run"] == nsteps
    assert np.array_equal(hist.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(ls.narrowband(w["nparts"]), nbs[-1])
    for k in ("fim_iters", "patch_visits", "check_visits", "nb_vertex_updates"):
        assert st[k] == ost[k], k


def _repartition(w, n, kind, size):
    w = dict(w)
    if kind == "block":
        w["npart"], w["nparts"] = synth.structured_partition(3, n + 1, size)
    else:
        w["npart"], w["nparts"] = lsgb300.partition_graph(3, w["elems"], len(w["xyz"]), size)
    return w


# graph partitions of 27 and 40 vertices and 4^3-vertex blocks: patches of up
# to 382, 481 and 672 element copies, i.e. the two-copies-per-thread sweep and
# the 512- and 1024-thread sweeps (one copy per thread), in both builds
@pytest.mark.parametrize("kind,size", [("graph", 27), ("graph", 40), ("block", 4)])
def test_large_patches_match_oracle(kind, size):
    n, nsteps = 14, 3
    w = _repartition(synth.workload("c3", n=n), n, kind, size)
    ex = lsgb300.from_workload(w, bit_exact=True)
    he, de = ex.solve(nsteps)
    ref, nbs, iters, ost = _oracle(w, False, 0.0, nsteps)
    assert de == ost["steps_run"] == nsteps
    assert np.array_equal(he.view(np.uint32), ref.view(np.uint32))
    st = ex.stats()
    for k in ("fim_iters", "patch_visits", "check_visits", "nb_vertex_updates"):
        assert st[k] == ost[k], k
    fast = lsgb300.from_workload(w)
    hf, df = fast.solve(nsteps)
    ref64, _, _, _ = _oracle(w, False, 0.0, nsteps, precision=64)
    assert df == nsteps
    for s in range(1, nsteps + 1):
        e, band = _band_err(hf[s], ref64[s], w)
        assert band.sum() > 0
        assert e.max() <= 1e-3, (s, e.max())


@pytest.mark.parametrize("name,n", [("c2", 9), ("c3", 14)])
@pytest.mark.parametrize("update", ["none", "advect", "curvature"])
def test_bitexact_update_kinds(name, n, update):
    w = synth.workload(name, n=n)
    w["update"] = update
    ls = lsgb300.from_workload(w, bit_exact=True)
    hist, done = ls.solve(3)
    ref, nbs, iters, ost = _oracle(w, False, 0.0, 3)
    assert done == ost["steps_run"] >= 1
    assert np.array_equal(hist.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("name,n", CASES)
@pytest.mark.parametrize("ctas,ref_compat", [(3, False), (5, False), (5, True)])
def test_fast_build_matches_oracle(name, n, ctas, ref_compat):
    # ref_compat: the reference's absolute SMALLNUM at unit-cube scale, where
    # even its FP32 and FP64 results lie up to ~0.5 h apart at a few vertices;
    # the bar is the same share of band vertices within 1e-3 h of the FP32
    # oracle
    w = synth.workload(name, n=n)
    nsteps = 3
    ls = lsgb300.from_workload(w, fim_ctas_per_sm=ctas, ref_compat=ref_compat)
    hist, done = ls.solve(nsteps)
    st = ls.stats()
    ref, nbs, iters, ost = _oracle(w, ref_compat, 0.0, nsteps)
    assert done == nsteps
    for s in range(1, nsteps + 1):
        e, band = _band_err(hist[s], ref[s], w)
        assert band.sum() > 0
        assert np.mean(e <= 1e-3) >= 0.98, (s, np.mean(e <= 1e-3), e.max())
    assert abs(st["nb_vertex_updates"] - ost["nb_vertex_updates"]) <= 0.005 * ost["nb_vertex_updates"]


@pytest.mark.parametrize("name,n,update", [("c3", 14, None), ("c2", 9, None), ("c3", 18, "none")])
def test_two_copies_per_thread_sweep_equals_one_copy_sweep(name, n, update):
    # fim_ctas_per_sm 5 runs the tet sweep with two element copies per thread
    # (state in shared memory); the solves, their listing and the per-vertex
    # minimum are the same, so the results and the work counters are equal
    w = synth.workload(name, n=n)
    if update:
        w["update"] = update
    # (6: the same kernel at six CTAs per SM; 7: with one copy per thread)
    nsteps = 4
    runs = []
    for ctas in (3, 5, 6, 7):
        ls = lsgb300.from_workload(w, fim_ctas_per_sm=ctas)
        hist, done = ls.solve(nsteps)
        runs.append((hist, done, ls.stats()))
    h3, d3, s3 = runs[0]
    for h5, d5, s5 in runs[1:]:
        assert d3 == d5 == nsteps
        assert np.array_equal(h3, h5)
        for key in ("fim_iters", "patch_visits", "check_visits", "nb_vertex_updates"):
            assert s3[key] == s5[key], key


def test_visits_run_by_checks_change_nothing():
    # on a mesh whose neighbour-check launches hold four or more patches per
    # resident CTA, the two-copies-per-thread kernel runs the visits of the
    # patches its checks activate in the same launch; the one-copy kernel
    # visits them in the next iteration: same bits, same work counters
    w = synth.workload("c3", n=128)
    nsteps = 2
    runs = {}
    for ctas in (3, 5):
        ls = lsgb300.from_workload(w, fim_ctas_per_sm=ctas)
        ls.step(nsteps)
        runs[ctas] = (ls.phi(), ls.stats())
    (p3, s3), (p5, s5) = runs[3], runs[5]
    assert s5["early_visits"] > 0 and s3["early_visits"] == 0
    assert s5["early_visits"] < s5["patch_visits"]
    assert np.array_equal(p3, p5)
    for key in ("fim_iters", "patch_visits", "check_visits", "nb_vertex_updates"):
        assert s3[key] == s5[key], key


@pytest.mark.parametrize("update", ["none", "curvature"])
def test_precision_form_meets_fp64_bar(update):
    # the metric's accuracy bar, max |phi - phi_FP64| <= 1e-3 h against the
    # oracle run in FP64, met by the precision form (the reference's solver
    # with FP64 repeats) and by the plain fast build (the planar-wave solver)
    w = synth.workload("c3", n=24)
    w["update"] = update
    nsteps = 3
    ref, _, _, _ = _oracle(w, False, 0.0, nsteps, precision=64)
    prec = lsgb300.from_workload(w, fp64_flagged=True)
    hp, _ = prec.solve(nsteps)
    plain = lsgb300.from_workload(w)
    hf, _ = plain.solve(nsteps)
    for s in range(1, nsteps + 1):
        e, _ = _band_err(hp[s], ref[s], w)
        assert e.max() <= 1e-3, (s, e.max())
        e, _ = _band_err(hf[s], ref[s], w)
        assert e.max() <= 1e-3, (s, e.max())
    assert prec.stats()["flagged_copies"] > 0


@pytest.mark.parametrize("name,n,update,nsteps", [("c3", 20, "curvature", 4), ("c3", 28, "none", 2),
                                                  ("c2", 16, "none", 2), ("c2", 12, "advect", 6)])
def test_fast_build_meets_fp64_bar(name, n, update, nsteps):
    # plain FP32 fast build against the oracle run in FP64 (every operation in
    # double): the planar-wave tet solver has no cancelling discriminant, so
    # the redistance stays at the FP64 result; the bar is 1e-3 h, the
    # reference's FP32 solver misses it by up to ~1e-1 h on these inputs
    w = synth.workload(name, n=n)
    w["update"] = update
    ref, _, _, _ = _oracle(w, False, 0.0, nsteps, precision=64)
    ls = lsgb300.from_workload(w)
    hist, done = ls.solve(nsteps)
    assert done == nsteps
    for s in range(1, nsteps + 1):
        e, band = _band_err(hist[s], ref[s], w)
        assert band.sum() > 0
        assert e.max() <= 1e-3, (s, e.max())


@pytest.mark.parametrize("staging", [False, True])
@pytest.mark.parametrize("offset", [0, 1])
def test_step_host_equals_device_steps(staging, offset):
    """ls_step_host through direct pageable access (where the GPU has it) or
    pinned staging, with 16-byte aligned and unaligned host arrays."""
    w = synth.workload("c2", n=9)
    a = lsgb300.from_workload(w)
    b = lsgb300.from_workload(w, flags=lsgb300.HOST_STAGING) if staging else lsgb300.from_workload(w)
    a.step(3)
    nv = len(w["phi0"])
    buf_a = np.zeros(nv + 4, np.float32)
    buf_b = np.zeros(nv + 4, np.float32)
    phi = buf_a[offset:offset + nv]
    out = buf_b[offset:offset + nv]
    phi[:] = w["phi0"]
    for _ in range(3):
        b.step_host(phi, out)
        phi, out = out, phi
    np.testing.assert_array_equal(a.phi(), phi)
    assert b.stats()["nb_vertex_updates"] == a.stats()["nb_vertex_updates"]


def test_graph_and_launch_paths_agree():
    w = synth.workload("c3", n=12)
    a = lsgb300.from_workload(w)
    b = lsgb300.from_workload(w, profile=True)
    ha, _ = a.solve(3)
    hb, _ = b.solve(3)
    np.testing.assert_array_equal(ha, hb)
    sb = b.stats()
    assert sb["n_sweep"] > 0 and sb["ms_sweep"] > 0


def test_profiled_launch_counts_belong_to_their_handle():
    # profiled kernel times are kept per handle and read when stats are asked
    # for: two handles stepped in turn report what each reports alone, and a
    # reset drops times that were not read yet
    keys = ("n_sweep", "n_check", "n_schedule", "n_seed", "n_narrowband", "n_update", "fim_iters", "patch_visits")
    wa, wb = synth.workload("c3", n=12), synth.workload("c2", n=10)
    alone = {}
    for name, w in (("a", wa), ("b", wb)):
        ls = lsgb300.from_workload(w, profile=True)
        ls.step(2)
        alone[name] = {k: ls.stats()[k] for k in keys}
    a = lsgb300.from_workload(wa, profile=True)
    b = lsgb300.from_workload(wb, profile=True)
    for _ in range(2):
        a.step(1)
        b.step(1)
    assert {k: a.stats()[k] for k in keys} == alone["a"]
    assert {k: b.stats()[k] for k in keys} == alone["b"]
    a.step(1)
    a.reset_stats()
    sa = a.stats()
    assert sa["n_sweep"] == 0 and sa["ms_sweep"] == 0 and sa["patch_visits"] == 0


def test_history_row0_is_phi0_and_default_inputs():
    w = synth.workload("c2", n=6)
    ls = lsgb300.from_workload(w)
    hist, done = ls.solve(2)
    np.testing.assert_array_equal(hist[0], w["phi0"])
    # defaults when phi / velocity are not given: phi0 = x - midX,
    # velocity (rangeX/100, 0, 0) (LevelSet.cu:221-233)
    p = lsgb300.default_params(bandwidth=w["bandwidth"], time_step=w["dt"])
    d = lsgb300.LevelSet(False, p)
    d.set_mesh(w["xyz"], w["elems"])
    d.set_partition(w["npart"], w["nparts"])
    d.setup()
    h, _ = d.solve(1)
    x = w["xyz"][:, 0].astype(np.float64)
    np.testing.assert_allclose(h[0], x - 0.5, atol=1e-6)


def test_empty_narrowband_stops_like_reference():
    w = synth.workload("c2", n=6)
    w["phi0"] = np.ones_like(w["phi0"])  # no interface: no seeds, empty band
    ls = lsgb300.from_workload(w)
    hist, done = ls.solve(3)
    assert done == 0 and len(hist) == 1


def test_fim_iteration_cap_reports_timeout():
    w = synth.workload("c3", n=12)
    ls = lsgb300.from_workload(w, max_fim_iters=2, graph_chunk=2)
    with pytest.raises(lsgb300.LevelSetError) as e:
        ls.solve(1)
    assert e.value.code == lsgb300.LS_DEVICE_TIMEOUT


@pytest.mark.parametrize("flags", [0, lsgb300.NO_GRAPH])
def test_slab_copy_wait_runs_out(flags):
    # a negative wait limit makes every slab wait of the two-copies sweep give
    # up at its first check: each CTA waits once more for its copies in
    # flight, leaves, and the step reports LS_DEVICE_TIMEOUT; the handle then
    # steps from phi0 with the normal limit and matches a fresh handle
    w = synth.workload("c3", n=16)
    ls = lsgb300.from_workload(w, flags=flags, barrier_wait_limit=-1)
    with pytest.raises(lsgb300.LevelSetError) as e:
        ls.step(1)
    assert e.value.code == lsgb300.LS_DEVICE_TIMEOUT
    p = ls.get_params()
    p.barrier_wait_limit = 0
    ls.set_params(p)
    ls.setup()
    ls.set_phi(w["phi0"])
    h1, d1 = ls.solve(2)
    h0, d0 = lsgb300.from_workload(w, flags=flags).solve(2)
    assert d0 == d1 == 2
    assert np.array_equal(h0.view(np.uint32), h1.view(np.uint32))


@pytest.mark.parametrize("flags", [0, lsgb300.PERSISTENT])
def test_launch_log_sums_to_profiled_totals(flags):
    # per-launch records of the profiled FIM launches: as many as the
    # profiled sweep and check launches, their times and algorithmic bytes
    # summing to the stats' totals
    w = synth.workload("c3", n=20)
    ls = lsgb300.from_workload(w, flags=flags)
    ls.step(1)
    ls.set_profile(True)
    ls.reset_stats()
    ls.step(2)
    kinds, ms, nbytes = ls.launch_log()
    st = ls.stats()
    assert len(kinds) == st["n_sweep"] + st["n_check"] > 0
    assert (kinds == 0).sum() == st["n_sweep"] and (kinds == 1).sum() == st["n_check"]
    assert (nbytes >= 0).all() and nbytes.sum() == st["sweep_slab_bytes"]
    assert abs(ms.sum() - (st["ms_sweep"] + st["ms_check"])) < 1e-3 * max(1.0, ms.sum())
    ls.reset_stats()
    assert len(ls.launch_log()[0]) == 0
