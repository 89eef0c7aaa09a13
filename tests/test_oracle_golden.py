"""The oracle is pinned to the reference: its local solvers and its host
curvature update reproduce the reference's own code (compiled from the
reference sources into oracle/_ref; outputs committed in tests/golden/)."""
import os

import numpy as np

import lsoracle
import synth

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_tet_solver_fp32_bit_exact():
    g = np.load(os.path.join(GOLD, "tet_solver.npz"))
    L = lsoracle.lib()
    sm, ln = float(g["smallnum"]), float(g["largenum"])
    out = np.array([L.lso_tet_solve_f32(*map(float, t), *map(float, m), sm, ln) for t, m in zip(g["T"], g["M"])],
                   np.float32)
    assert np.array_equal(out.view(np.uint32), g["out32"].view(np.uint32))


def test_tet_solver_fp64_bit_exact():
    g = np.load(os.path.join(GOLD, "tet_solver.npz"))
    L = lsoracle.lib()
    sm, ln = float(g["smallnum"]), float(g["largenum"])
    out = np.array([L.lso_tet_solve_f64(*map(float, t), *map(float, m), sm, ln) for t, m in zip(g["T"], g["M"])])
    assert np.array_equal(out, g["out64"])


def test_tri_solver_fp64_bit_exact():
    g = np.load(os.path.join(GOLD, "tri_solver.npz"))
    L = lsoracle.lib()
    out = np.array([L.lso_tri_solve_f64(t[0], t[1], *l, 1e9) for t, l in zip(g["T"], g["L"])])
    assert np.array_equal(out, g["out"])


def test_curvature_update_matches_reference_host_function():
    g = np.load(os.path.join(GOLD, "curvature_step.npz"))
    xyz, tets, phi, dt, out = g["xyz"], g["tets"], g["phi"], float(g["dt"]), g["out"]
    npart, nparts = synth.structured_partition(3, 5, 3)
    ol = lsoracle.OracleLayout(3, xyz, tets, npart, nparts)
    p = ol.params(update_kind=1, dt=dt, curv_coeff=1.0, ref_compat=1, bandwidth=100.0)
    mine = ol.update_only(p, phi, None, np.arange(nparts))
    # same formula; the per-vertex sums run in a different element order
    moved = np.abs(out - phi)
    assert moved.max() > 1e-3
    np.testing.assert_allclose(mine, out, rtol=0, atol=2e-6 * max(1.0, float(np.abs(out).max())))
