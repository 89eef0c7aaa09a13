"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs only where the reference tree is present and oracle/_ref has been built
(python oracle/build_ref.py): the reference's own local solvers and host
curvature update, compiled from its sources, are evaluated on seeded inputs
and their outputs saved as small .npz fixtures.  The tests compare the
oracle against these files, so that a machine without the reference tree
also checks the oracle against the reference.

    python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref")
sys.path.insert(0, os.path.join(ROOT, "sci-solver_level-set_gb300"))
import synth  # noqa: E402

F, D, I, V = ctypes.c_float, ctypes.c_double, ctypes.c_int, ctypes.c_void_p


def tet_metric(P):
    """FP32 local coordinates and metric terms of a tet, in the order and
    arithmetic the FIM kernel forms them (redistance_kernels3d.h:379-396)."""
    P = P.astype(np.float32)
    AB, AC, AD = P[1] - P[0], P[2] - P[0], P[3] - P[0]
    lenAB = np.float32(np.sqrt(np.float32(AB @ AB)))
    N = np.cross(AB, AC).astype(np.float32)
    Z = N / np.float32(np.sqrt(np.float32(N @ N)))
    X = AB / lenAB
    Y = np.cross(Z, X).astype(np.float32)
    L = [np.float32(v) for v in (lenAB, AC @ X, AC @ Y, AD @ X, AD @ Y, AD @ Z)]
    ACBC = L[1] * (L[1] - L[0]) + L[2] * L[2]
    BCCD = (L[1] - L[0]) * (L[3] - L[1]) + L[2] * (L[4] - L[2])
    ACCD = L[1] * (L[3] - L[1]) + L[2] * (L[4] - L[2])
    ADBD = L[3] * (L[3] - L[0]) + L[4] * L[4] + L[5] * L[5]
    ACAD = L[1] * L[3] + L[2] * L[4]
    BCBD = (L[1] - L[0]) * (L[3] - L[0]) + L[2] * L[4]
    ADBC = ACBC + BCCD
    ACBD = ACBC + ACCD
    CDBD = ADBD - ACBD
    ADCD = ADBD - ADBC
    CDCD = ADCD - ACCD
    ACAC = ACAD - ACCD
    BCBC = BCBD - BCCD
    return np.array([ACAC, ACBC, ACCD, BCBC, BCCD, CDCD], np.float32)


def solver_inputs(n, seed):
    """Seeded tets (unit cell corners, jittered, random vertex order, scales
    1e-2..10) with arrival times from plane waves and point sources, plus a
    share of LARGENUM (unreached) values."""
    rng = np.random.default_rng(seed)
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [1, 1, 1]], float)
    T = np.zeros((n, 3), np.float32)
    M = np.zeros((n, 6), np.float32)
    i = 0
    while i < n:
        s = 10 ** rng.uniform(-2, 1)
        P = (base[rng.permutation(4)] + rng.uniform(-0.3, 0.3, (4, 3))) * s
        if rng.random() < 0.5:
            nrm = rng.normal(size=3)
            nrm /= np.linalg.norm(nrm)
            t = P @ nrm + rng.uniform(0, 5) * s
        else:
            c = P[0] + rng.normal(size=3) * rng.uniform(1, 6) * s
            t = np.linalg.norm(P - c, axis=1)
        if (t[:3] < 0).any():
            continue
        t = t[:3].astype(np.float32)
        if rng.random() < 0.05:
            t[rng.integers(3)] = 1e9
        T[i] = t
        M[i] = tet_metric(P)
        i += 1
    return T, M


def main():
    tet = ctypes.CDLL(os.path.join(REF, "libref_tet.so"))
    tri = ctypes.CDLL(os.path.join(REF, "libref_tri.so"))
    k20 = ctypes.CDLL(os.path.join(REF, "libref_k20.so"))
    tet.lsref_tet_solve_f32.restype = F
    tet.lsref_tet_solve_f32.argtypes = [F] * 9
    tet.lsref_smallnum.restype = D
    tet.lsref_largenum.restype = D
    tri.lsref_tri_solve_f64.restype = D
    tri.lsref_tri_solve_f64.argtypes = [D] * 5
    tri.lsref_tet_solve_f64.restype = D
    tri.lsref_tet_solve_f64.argtypes = [D] * 9
    k20.lsref_curvature_step.restype = I
    k20.lsref_curvature_step.argtypes = [I, V, I, V, V, I, F, V]

    # 1. tet local solver, FP32 (3D stack) and FP64 (2D stack's copy)
    T, M = solver_inputs(4000, 1)
    out32 = np.array([tet.lsref_tet_solve_f32(*map(float, t), *map(float, m)) for t, m in zip(T, M)], np.float32)
    out64 = np.array([tri.lsref_tet_solve_f64(*map(float, t), *map(float, m)) for t, m in zip(T, M)], np.float64)
    np.savez_compressed(os.path.join(HERE, "tet_solver.npz"), T=T, M=M, out32=out32, out64=out64,
                        smallnum=tet.lsref_smallnum(), largenum=tet.lsref_largenum())
    # 2. triangle local solver, FP64
    rng = np.random.default_rng(2)
    n = 4000
    TT = np.zeros((n, 2))
    LL = np.zeros((n, 3))
    for i in range(n):
        s = 10 ** rng.uniform(-2, 1)
        P = rng.uniform(0, 1, (3, 2)) * s
        LL[i] = [np.linalg.norm(P[1] - P[0]), np.linalg.norm(P[2] - P[1]), np.linalg.norm(P[2] - P[0])]
        c = P[0] + rng.normal(size=2) * s * 3
        TT[i] = [np.linalg.norm(P[0] - c), np.linalg.norm(P[1] - c)]
        if rng.random() < 0.05:
            TT[i, rng.integers(2)] = 1e9
    outtri = np.array([tri.lsref_tri_solve_f64(TT[i, 0], TT[i, 1], *LL[i]) for i in range(n)])
    np.savez_compressed(os.path.join(HERE, "tri_solver.npz"), T=TT, L=LL, out=outtri)
    # 3. host mean-curvature update (meshFIM3d::updateT_single_stage) on a
    #    small jittered cube, all elements in the narrowband, h ~ 1 frame
    xyz, tets = synth.cube_mesh(4, 0.15, seed=3, scale=4.0)
    phi = synth.phi_spheres(xyz, [(2.0, 2.0, 2.0)], [1.3])
    dt = np.float32(0.1)
    out = phi.copy()
    nb = np.arange(len(tets), dtype=np.int32)
    k20.lsref_curvature_step(len(xyz), xyz.ctypes.data, len(tets), np.ascontiguousarray(tets).ctypes.data,
                             nb.ctypes.data, len(nb), dt, out.ctypes.data)
    np.savez_compressed(os.path.join(HERE, "curvature_step.npz"), xyz=xyz, tets=tets, phi=phi, dt=dt, out=out)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
