"""The fast build's planar-wave tet solver (tet_solve_wave in
csrc/ls_device.cuh), restated here in float64 numpy, against the oracle's
FP64 restatement of the reference's local solver
(src/core3d/include/redistance_kernels3d.h:124-285) on jittered-lattice tets
with eikonal-consistent arrival times.  In exact arithmetic the two compute
the same minimum over the same candidates; in float64 they agree to ~1e-11,
and the float32 form of the wave solver stays within ~5e-5 h of the FP64
reference where the reference's own float32 form is up to ~0.3 h off (its
discriminants cancel).  CPU only: the kernels are checked against FP64 on the
GPU by tests/test_gpu_parity.py."""
import numpy as np
import pytest

import lsoracle


def _metric(P):
    A, B, C, D = P[:, 0], P[:, 1], P[:, 2], P[:, 3]
    AC, BC, CD = C - A, C - B, D - C
    dot = lambda x, y: (x * y).sum(1)
    return [dot(AC, AC), dot(AC, BC), dot(AC, CD), dot(BC, BC), dot(BC, CD), dot(CD, CD)]


def wave(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps, dt=np.float64):
    """tet_solve_wave, vectorised: edges; the three sides from the planar
    wave, each with its distance |f x w| / sqrt(|f|^2 - u^2) at the
    stationary point; the interior root and its mirror with the reference's
    l2 = (s l1 + t) / (h + eps), each evaluated at its point."""
    one, eps = dt(1), dt(eps)
    with np.errstate(all="ignore"):
        best = np.minimum(np.minimum(TA + np.sqrt((ACAC + ACCD) + (ACCD + CDCD)),
                                     TB + np.sqrt((BCBC + BCCD) + (BCCD + CDCD))), TC + np.sqrt(CDCD))

        def side(TP, TQ, ff, fw, ww):
            u = TQ - TP
            r = np.sqrt(ff * ww - fw * fw) / np.sqrt(ff - u * u)
            lam = (fw - u * r) / ff
            ok = (lam >= 0) & (lam <= 1)
            return np.where(ok, TP + lam * u + r, np.inf)

        best = np.fmin(best, side(TC, TB, BCBC, -BCCD, CDCD))
        best = np.fmin(best, side(TC, TA, ACAC, -ACCD, CDCD))
        ff = (BCBC - ACBC) + (ACAC - ACBC)
        fw = (BCBC + BCCD) - (ACBC + ACCD)
        ww = (BCBC + BCCD) + (BCCD + CDCD)
        best = np.fmin(best, side(TB, TA, ff, fw, ww))
        u1, u2 = TA - TC, TB - TC
        idet = one / (ACAC * BCBC - ACBC * ACBC)
        g1 = (BCBC * u1 - ACBC * u2) * idet
        g2 = (ACAC * u2 - ACBC * u1) * idet
        foot1 = (ACBC * BCCD - BCBC * ACCD) * idet
        det3 = (ACAC * (BCBC * CDCD - BCCD * BCCD) - ACBC * (ACBC * CDCD - BCCD * ACCD) +
                ACCD * (ACBC * BCCD - BCBC * ACCD))
        hD = np.sqrt(np.maximum(det3 * idet, 0))
        dl = hD / np.sqrt(one - (g1 * u1 + g2 * u2)) * g1
        TAC, TBC = TC - TA, TC - TB
        s = TAC * ACBC - TBC * ACAC
        t = TAC * BCCD - TBC * ACCD
        h = -(TAC * BCBC - TBC * ACBC)
        for l1 in (foot1 - dl, foot1 + dl):
            l2 = (s * l1 + t) / (h + eps)
            l3 = one - l1 - l2
            ok = (l1 >= 0) & (l1 <= 1) & (l2 >= 0) & (l2 <= 1) & (l3 >= 0) & (l3 <= 1)
            c = TA * l1 + TB * l2 + TC * l3 + np.sqrt((l1 * ACAC + l2 * ACBC + ACCD) * l1 +
                                                      (l1 * ACBC + l2 * BCBC + BCCD) * l2 + (l1 * ACCD + l2 * BCCD + CDCD))
            best = np.fmin(best, np.where(ok, c, np.inf))
    return best


def _cases(family, n=20000, seed=1):
    """Tets of a jittered 64^3 Freudenthal lattice (random vertex order, the
    last vertex the target) in the scaled frame (h = 1), arrival times from a
    sphere, an axis-aligned plane, a random plane or a noisy sphere."""
    rng = np.random.default_rng(seed)
    m, h = 64, 1.0 / 64
    base = rng.integers(1, m - 2, size=(n, 3)).astype(np.float64)
    perm = np.array([[0, 1, 2], [0, 2, 1], [1, 0, 2], [1, 2, 0], [2, 0, 1], [2, 1, 0]])[rng.integers(0, 6, n)]
    V = np.zeros((n, 4, 3))
    V[:, 0] = base
    cur = base.copy()
    for j in range(3):
        step = np.zeros((n, 3))
        step[np.arange(n), perm[:, j]] = 1
        cur = cur + step
        V[:, j + 1] = cur
    V = V * h + rng.uniform(-0.15 * h, 0.15 * h, size=V.shape)
    order = np.argsort(rng.random((n, 4)), axis=1)
    V = np.take_along_axis(V, order[:, :, None], axis=1)
    if family == "sphere":
        c = rng.uniform(0.2, 0.8, size=(n, 1, 3))
        T = np.linalg.norm(V - c, axis=2) - rng.uniform(0.05, 0.3, size=(n, 1))
    elif family == "plane_axis":
        ax = rng.integers(0, 3, n)
        T = V[np.arange(n)[:, None], np.arange(4)[None, :], ax[:, None]] - rng.uniform(0, 1, (n, 1))
    elif family == "plane_rand":
        nv = rng.normal(size=(n, 1, 3))
        nv /= np.linalg.norm(nv, axis=2, keepdims=True)
        T = (V * nv).sum(2) - rng.uniform(-1, 1, (n, 1))
    else:
        c = rng.uniform(0.2, 0.8, size=(n, 1, 3))
        T = np.linalg.norm(V - c, axis=2) + rng.uniform(-0.3, 0.3, (n, 4)) * h
    T = np.abs(T) / h
    M = _metric(V / h)
    return T[:, 0], T[:, 1], T[:, 2], M


def _reference(TA, TB, TC, M, precision):
    L = lsoracle.lib()
    f = L.lso_tet_solve_f64 if precision == 64 else L.lso_tet_solve_f32
    cast = float if precision == 64 else (lambda x: float(np.float32(x)))
    return np.array([f(*[cast(x) for x in (TA[i], TB[i], TC[i], *(m[i] for m in M))], 1e-5, 1e9)
                     for i in range(len(TA))])


FAMILIES = ["sphere", "plane_axis", "plane_rand", "noisy_sphere"]


@pytest.mark.parametrize("family", FAMILIES)
def test_wave_form_equals_reference_solver_in_fp64(family):
    TA, TB, TC, M = _cases(family)
    ref64 = _reference(TA, TB, TC, M, 64)
    w64 = wave(TA, TB, TC, *M, 1e-5)
    assert np.all(np.isfinite(w64))
    assert np.abs(w64 - ref64).max() <= 1e-9


def test_wave_form_in_fp32_stays_at_fp64_where_the_reference_form_does_not():
    worst_wave, worst_ref = 0.0, 0.0
    for family in FAMILIES:
        TA, TB, TC, M = _cases(family, seed=2)
        ref64 = _reference(TA, TB, TC, M, 64)
        ref32 = _reference(TA, TB, TC, M, 32)
        w32 = wave(*[np.asarray(a, np.float32) for a in (TA, TB, TC, *M)], 1e-5, dt=np.float32).astype(np.float64)
        worst_wave = max(worst_wave, np.abs(w32 - ref64).max())
        worst_ref = max(worst_ref, np.abs(ref32 - ref64).max())
    # values in units of h: the wave form's FP32 error stays ~1e-5 h, the
    # reference form's FP32 loses candidates to cancelled discriminants
    assert worst_wave <= 1e-4, worst_wave
    assert worst_ref >= 1e-2, worst_ref
