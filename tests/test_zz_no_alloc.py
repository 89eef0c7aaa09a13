"""The narrowband entry point that allocates no device memory.

ls_narrowband_noalloc serves callers that cannot call cudaMalloc: host
applications that own all device memory through their own pool, or that run
under a fixed device-memory budget, where an allocation inside the call would
take memory already handed out or fail.  They pass their own device buffers
and the kernel's scratch lives in a fixed device array inside the library.
These tests compare it, through the C ABI, with the solver's own narrowband
selection for the same step, on two calls in a row, once in the caller's
units (FIM scale 1) and once in a scaled FIM frame where far vertices keep
DT = largenum (all three phi formulas).  (The device buffers here are
allocated by the test, as such a caller would.)
"""
import ctypes

import numpy as np
import pytest

import lsgb300
import synth

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _call(torch, L, nv, nparts, d_off, d_dt, d_sign, bandwidth, scale, largenum):
    d_phi = torch.full((nv,), float("nan"), dtype=torch.float32, device="cuda")
    d_flags = torch.full((nparts,), 7, dtype=torch.uint8, device="cuda")
    counts = np.zeros(3, np.int64)
    torch.cuda.synchronize()
    rc = L.ls_narrowband_noalloc(nv, nparts, d_off.data_ptr(), d_dt.data_ptr(), d_sign.data_ptr(),
                                 ctypes.c_float(bandwidth), ctypes.c_float(scale), ctypes.c_float(largenum),
                                 d_phi.data_ptr(), d_flags.data_ptr(), counts.ctypes.data, None)
    return rc, d_phi.cpu().numpy(), d_flags.cpu().numpy(), counts


def _compare_with_solver(ls, w, bandwidth_fim, scale, largenum):
    torch = pytest.importorskip("torch")
    hist, done = ls.solve(1)
    assert done == 1
    ref_phi = hist[1]
    ref_flags = ls.narrowband(w["nparts"])
    st = ls.stats()
    _, dt = ls.debug_active(with_dt=True)          # layout vertex order
    vperm = ls.layout("vert_permute")
    voff = ls.layout("vert_offsets")
    sign = (w["phi0"][vperm] >= 0).astype(np.uint8)
    nv, nparts = len(dt), w["nparts"]
    d_off, d_dt, d_sign = _dev(torch, voff), _dev(torch, dt), _dev(torch, sign)
    L = lsgb300.lib()
    for call in range(2):
        rc, phi_new, flags, counts = _call(torch, L, nv, nparts, d_off, d_dt, d_sign, bandwidth_fim, scale,
                                           largenum)
        assert rc == lsgb300.LS_OK, call
        phi = np.empty_like(phi_new)
        phi[vperm] = phi_new                       # caller's vertex order
        np.testing.assert_array_equal(phi, ref_phi)
        np.testing.assert_array_equal(flags, ref_flags)
        assert counts[0] == st["nb_patches"], call
        assert counts[1] == st["nb_vertex_updates"], call
        assert counts[2] == st["nb_patch_vertices"], call
    return dt


def test_narrowband_noalloc_matches_solver_two_calls():
    w = synth.workload("c3", n=24)
    w["update"] = "none"
    # the reference's semantics keep the FIM frame in the caller's units
    # (scale 1), so the inputs below are exactly the solver's
    ls = lsgb300.from_workload(w, ref_compat=True)
    _compare_with_solver(ls, w, w["bandwidth"], 1.0, 1e9)


def test_narrowband_noalloc_scaled_frame_and_far_vertices():
    # FIM frame with length unit h: phi = +-DT * h inside the FIM's reach and
    # +-largenum outside it; bandwidth in that frame is w / h
    w = synth.workload("c3", n=24)
    w["update"] = "none"
    h = float(w["h"])
    ls = lsgb300.from_workload(w, length_scale=h)
    dt = _compare_with_solver(ls, w, float(np.float32(w["bandwidth"] / h)), float(np.float32(h)), 1e9)
    assert np.any(dt >= 1e9) and np.any(dt < 1e9)


def test_narrowband_noalloc_negative_and_signed_zero_dt():
    # values below +0 rank as floats: a patch whose only in-band values are
    # -0.0 or negative is still selected
    torch = pytest.importorskip("torch")
    voff = np.array([0, 3, 6, 9], np.int32)
    dt = np.array([5.0, 6.0, -0.0, 7.0, -2.0, 8.0, 9.0, 9.5, 9.9], np.float32)
    sign = np.ones(9, np.uint8)
    L = lsgb300.lib()
    for call in range(2):
        rc, phi, flags, counts = _call(torch, L, 9, 3, _dev(torch, voff), _dev(torch, dt), _dev(torch, sign),
                                       1.0, 1.0, 1e9)
        assert rc == lsgb300.LS_OK
        np.testing.assert_array_equal(flags, [1, 1, 0])
        np.testing.assert_array_equal(phi.view(np.uint32), dt.view(np.uint32))
        assert list(counts) == [2, 2, 6], call


def test_narrowband_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    small = torch.zeros(16, dtype=torch.int32, device="cuda")
    counts = np.zeros(3, np.int64)
    p = small.data_ptr()
    rc = lsgb300.lib().ls_narrowband_noalloc(4, (1 << 20) + 1, p, p, p, ctypes.c_float(1.0), ctypes.c_float(1.0),
                                             ctypes.c_float(1e9), p, p, counts.ctypes.data, None)
    assert rc == lsgb300.LS_BAD_INPUT
