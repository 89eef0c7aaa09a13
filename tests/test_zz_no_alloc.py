"""The narrowband entry point that allocates no device memory.

ls_narrowband_noalloc serves callers that cannot call cudaMalloc (host
applications that own all device memory through their own pool, fixed
memory budgets, steps recorded once and replayed): they pass their own device
buffers and the kernel's scratch lives in a fixed device array inside the
library.  This test compares it, through the C ABI, with the solver's own
narrowband selection for the same step, on two calls in a row.  (The device
buffers here are allocated by the test, as such a caller would.)
"""
import ctypes

import numpy as np
import pytest

import lsgb300
import synth

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_narrowband_noalloc_matches_solver_two_calls():
    torch = pytest.importorskip("torch")
    w = synth.workload("c3", n=24)
    w["update"] = "none"
    # the reference's semantics keep the FIM frame in the caller's units
    # (scale 1), so the inputs below are exactly the solver's
    ls = lsgb300.from_workload(w, ref_compat=True)
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
        d_phi = torch.full((nv,), float("nan"), dtype=torch.float32, device="cuda")
        d_flags = torch.full((nparts,), 7, dtype=torch.uint8, device="cuda")
        counts = np.zeros(3, np.int64)
        torch.cuda.synchronize()
        rc = L.ls_narrowband_noalloc(nv, nparts, d_off.data_ptr(), d_dt.data_ptr(), d_sign.data_ptr(),
                                     ctypes.c_float(w["bandwidth"]), ctypes.c_float(1.0), ctypes.c_float(1e9),
                                     d_phi.data_ptr(), d_flags.data_ptr(), counts.ctypes.data, None)
        assert rc == lsgb300.LS_OK, call
        phi_new = d_phi.cpu().numpy()
        phi = np.empty_like(phi_new)
        phi[vperm] = phi_new                       # caller's vertex order
        np.testing.assert_array_equal(phi, ref_phi)
        np.testing.assert_array_equal(d_flags.cpu().numpy(), ref_flags)
        assert counts[0] == st["nb_patches"], call
        assert counts[1] == st["nb_vertex_updates"], call
        assert counts[2] == st["nb_patch_vertices"], call


def test_narrowband_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    small = torch.zeros(16, dtype=torch.int32, device="cuda")
    counts = np.zeros(3, np.int64)
    p = small.data_ptr()
    rc = lsgb300.lib().ls_narrowband_noalloc(4, (1 << 20) + 1, p, p, p, ctypes.c_float(1.0), ctypes.c_float(1.0),
                                             ctypes.c_float(1e9), p, p, counts.ctypes.data, None)
    assert rc == lsgb300.LS_BAD_INPUT
