"""The oracle and the product are pinned to the reference: the oracle's local
solvers and host curvature update reproduce the reference's own code; the
product's patch layout builder and the oracle's restatement of it reproduce
the layout the reference's own InitPatches / InitPatches2 /
GenerateBlockNeighbors build; and the oracle's time step reproduces the
reference's own meshFIM3d::GenerateData (seed search, FIM redistance with its
host-driven lists, narrowband, advection update) bit for bit.  The reference
pieces are compiled from its sources into oracle/_ref (its kernels run on the
CPU); their outputs are committed in tests/golden/."""
import hashlib
import os

import numpy as np
import pytest

import lsgb300
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


def _layout_cases():
    with np.load(os.path.join(GOLD, "ref_layout.npz")) as g:
        return [str(c) for c in g["cases"]]


class _Case:
    """One case's entries of the layout golden file, keyed without the case
    prefix."""

    def __init__(self, d):
        self._d = d
        self.files = list(d)

    def __getitem__(self, k):
        return self._d[k]


def _same(g, key, mine):
    """Bit-exact comparison with the stored array, or with its length and
    SHA-256 digest where only those are stored."""
    mine = np.ascontiguousarray(mine)
    if key in g.files:
        ref = g[key]
        if ref.dtype == np.float64:  # the 2D reference keeps local coordinates in double
            ref = ref.astype(np.float32)
        return mine.shape == ref.shape and np.array_equal(mine.view(np.uint8), ref.view(np.uint8))
    return (mine.size == int(g[key + ":len"]) and
            hashlib.sha256(mine.tobytes()).hexdigest() == str(g[key + ":sha256"]))


@pytest.mark.parametrize("case", _layout_cases())
def test_layout_equals_reference_layout(case):
    with np.load(os.path.join(GOLD, "ref_layout.npz")) as z:
        g = _Case({k.split(":", 1)[1]: z[k] for k in z.files if k.startswith(case + ":")})
    dim = int(g["dim"])
    xyz, el, npart, nparts = g["xyz"], g["elems"], g["npart"], int(g["nparts"])
    if int(g["side"]) > 0:
        # the reference's GraphPartition_Square labels = the structured partitioner's
        mine, n = lsgb300.partition_structured(dim, int(g["side"]), int(g["block"]), len(xyz))
        assert n == nparts and np.array_equal(mine, npart)
    ls = lsgb300.LevelSet(dim == 2)
    ls.set_mesh(xyz, el)
    ls.set_partition(npart, nparts)
    ls.prepare()
    info = ls.layout_info()
    assert info["nparts"] == nparts and info["full"] == int(g["full"]) and info["lep"] == int(g["lep"])
    ol = lsoracle.OracleLayout(dim, xyz, el, npart, nparts)
    for a in lsgb300.REF_ARRAYS:
        assert _same(g, a, ls.layout(a).ravel()), (case, "product", a)
        assert _same(g, a, ol.array(a).ravel()), (case, "oracle", a)


def _step_cases():
    with np.load(os.path.join(GOLD, "ref_steps.npz")) as g:
        return [str(c) for c in g["cases"]]


def load_step_case(case):
    """Inputs and phi history of one case of the reference's time steps."""
    with np.load(os.path.join(GOLD, "ref_steps.npz")) as z:
        return {k.split(":", 1)[1]: z[k] for k in z.files if k.startswith(case + ":")}


@pytest.mark.parametrize("case", _step_cases())
def test_oracle_equals_reference_time_steps(case):
    g = load_step_case(case)
    hist = g["history"]
    nsteps = len(hist) - 1
    ol = lsoracle.OracleLayout(3, g["xyz"], g["elems"], g["npart"], int(g["nparts"]))
    p = ol.params(update_kind=lsoracle.UPDATE["advect"], dt=float(g["dt"]), bandwidth=float(g["bandwidth"]),
                  curv_coeff=1.0, ref_compat=1)
    ref, _, _, ost = ol.solve(p, g["phi0"], g["vel"], nsteps)
    assert ost["steps_run"] == nsteps
    assert np.array_equal(ref.view(np.uint32), hist.view(np.uint32))
