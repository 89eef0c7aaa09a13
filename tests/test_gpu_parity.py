"""GPU parity: the sm_103a path through the C ABI against the CPU oracle on
the same seeded inputs (small members of the benchmark families).

Tolerances (floating point, per the BASELINE parity bar):
  * phi per step inside the narrowband: max |phi_gpu - phi_oracle| <= 1e-4 h
    with the precision form (tet solves whose discriminant cancels are
    repeated in FP64 on both sides);
  * plain FP32: at least 99.9% of band vertices within 1e-4 h (an FP32 solve
    with a cancelled discriminant can round differently under the GPU's
    fused multiply-adds than under the oracle's unfused arithmetic);
  * narrowband patch sets per step: identical;
  * vertex-update counts: identical.
"""
import numpy as np
import pytest

import lsgb300
import lsoracle
import synth

pytestmark = pytest.mark.gpu

CASES = [("c1", 16), ("c2", 9), ("c3", 16)]


def _oracle(w, ref_compat, tau, nsteps, precision=32):
    ol = lsoracle.OracleLayout(w["dim"], w["xyz"], w["elems"], w["npart"], w["nparts"])
    p = ol.params(update_kind=lsoracle.UPDATE[w["update"]], dt=w["dt"], bandwidth=w["bandwidth"],
                  curv_coeff=1.0, ref_compat=1 if ref_compat else 0, fp64_tau=tau, precision=precision)
    return ol.solve(p, w["phi0"], w["vel"], nsteps)


def _band_err(a, b, w):
    band = (np.abs(b) <= w["bandwidth"]) & (np.abs(a) <= w["bandwidth"])
    return np.abs(a[band] - b[band]) / w["h"], band


@pytest.mark.parametrize("name,n", CASES)
@pytest.mark.parametrize("ref_compat", [False, True])
def test_precision_form_matches_oracle(name, n, ref_compat):
    w = synth.workload(name, n=n)
    nsteps = 4
    tau = 2.0 ** -18 if w["dim"] == 3 else 0.0
    ls = lsgb300.from_workload(w, ref_compat=ref_compat, fp64_flagged=True)
    hist, done = ls.solve(nsteps)
    st = ls.stats()
    ref, nbs, iters, ost = _oracle(w, ref_compat, tau, nsteps)
    assert done == ost["steps_run"] == nsteps
    for s in range(1, nsteps + 1):
        e, band = _band_err(hist[s], ref[s], w)
        assert band.sum() > 0
        assert e.max() <= 1e-4, (s, e.max())
    assert st["nb_vertex_updates"] == ost["nb_vertex_updates"]
    assert st["nb_patches"] == ost["nb_patches"]
    nb = ls.narrowband(w["nparts"])
    assert np.array_equal(nb, nbs[-1])


@pytest.mark.parametrize("name,n", CASES)
def test_plain_fp32_matches_oracle(name, n):
    w = synth.workload(name, n=n)
    nsteps = 3
    ls = lsgb300.from_workload(w)
    hist, done = ls.solve(nsteps)
    ref, nbs, iters, ost = _oracle(w, False, 0.0, nsteps)
    assert done == nsteps
    for s in range(1, nsteps + 1):
        e, band = _band_err(hist[s], ref[s], w)
        assert np.mean(e <= 1e-4) >= 0.999, (s, np.mean(e <= 1e-4), e.max())


def test_precision_form_tracks_fp64_oracle():
    # the metric's accuracy bar: max |phi - phi_FP64| <= 1e-3 h
    w = synth.workload("c3", n=24)
    nsteps = 3
    ls = lsgb300.from_workload(w, fp64_flagged=True)
    hist, _ = ls.solve(nsteps)
    ref, _, _, _ = _oracle(w, False, 0.0, nsteps, precision=64)
    for s in range(1, nsteps + 1):
        e, band = _band_err(hist[s], ref[s], w)
        assert e.max() <= 1e-3, (s, e.max())


def test_step_host_equals_device_steps():
    w = synth.workload("c2", n=9)
    a = lsgb300.from_workload(w)
    b = lsgb300.from_workload(w)
    a.step(3)
    phi = w["phi0"].copy()
    out = np.empty_like(phi)
    for _ in range(3):
        b.step_host(phi, out)
        phi, out = out, phi
    np.testing.assert_array_equal(a.phi(), phi)


def test_graph_and_launch_paths_agree():
    w = synth.workload("c3", n=12)
    a = lsgb300.from_workload(w)
    b = lsgb300.from_workload(w, profile=True)
    ha, _ = a.solve(3)
    hb, _ = b.solve(3)
    np.testing.assert_array_equal(ha, hb)
    sb = b.stats()
    assert sb["n_sweep"] > 0 and sb["ms_sweep"] > 0


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
