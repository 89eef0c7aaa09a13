"""ctypes wrapper of the CPU oracle (oracle/build/liblsoracle.so).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline / reference legs use it as the checker.  The product library
never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liblsoracle.so")
SOURCES = ["lsoracle.c"]

ARRAYS = {
    "ele_permute": 0, "ele_offsets": 1, "vert_permute": 2, "vert_offsets": 3,
    "ele_after_permute": 4, "mem_locations": 5, "mem_location_offsets": 6,
    "block_xadj": 7, "block_adjncy": 8, "local_coords": 9, "vert_ipermute": 10,
}


def build():
    """Compile the oracle with gcc: no FP contraction, so x86 and Arm hosts
    give the same bits."""
    os.makedirs(os.path.join(HERE, "build"), exist_ok=True)
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11",
           "-o", LIB_PATH] + [os.path.join(HERE, s) for s in SOURCES] + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    return LIB_PATH


class Params(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("precision", ctypes.c_int), ("ref_compat", ctypes.c_int),
        ("update_kind", ctypes.c_int), ("niter", ctypes.c_int), ("inside_niter", ctypes.c_int),
        ("max_fim_iters", ctypes.c_int), ("nthreads", ctypes.c_int), ("dt", ctypes.c_double),
        ("bandwidth", ctypes.c_double), ("curv_coeff", ctypes.c_double), ("smallnum", ctypes.c_double),
        ("largenum", ctypes.c_double), ("length_scale", ctypes.c_double), ("fp64_tau", ctypes.c_double),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("steps_run", ctypes.c_int), ("status", ctypes.c_int), ("fim_iters", ctypes.c_longlong),
        ("patch_visits", ctypes.c_longlong), ("check_visits", ctypes.c_longlong),
        ("nb_vertex_updates", ctypes.c_longlong), ("nb_patch_vertices", ctypes.c_longlong),
        ("nb_patches", ctypes.c_longlong), ("seconds", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        V, I = ctypes.c_void_p, ctypes.c_int
        L.lso_layout_build.argtypes = [I, I, V, I, V, V, I, ctypes.POINTER(V)]
        L.lso_layout_info.argtypes = [V, V]
        L.lso_layout_copy.argtypes = [V, I, V]
        L.lso_layout_free.argtypes = [V]
        L.lso_solve.argtypes = [V, ctypes.POINTER(Params), V, V, I, V, V, V, ctypes.POINTER(Stats)]
        L.lso_update_only.argtypes = [V, ctypes.POINTER(Params), V, V, V, I, V]
        F, D = ctypes.c_float, ctypes.c_double
        L.lso_tet_solve_f32.restype = F
        L.lso_tet_solve_f32.argtypes = [F] * 9 + [D, F]
        L.lso_tet_solve_f64.restype = D
        L.lso_tet_solve_f64.argtypes = [D] * 9 + [D, D]
        L.lso_tri_solve_f64.restype = D
        L.lso_tri_solve_f64.argtypes = [D] * 5 + [D]
        L.lso_tri_solve_f32.restype = F
        L.lso_tri_solve_f32.argtypes = [F] * 5 + [F]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleLayout:
    def __init__(self, dim, xyz, elems, npart, nparts):
        self.dim = dim
        self._xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
        self._el = np.ascontiguousarray(elems, np.int32)
        self._np = np.ascontiguousarray(npart, np.int32)
        self._h = ctypes.c_void_p()
        rc = lib().lso_layout_build(dim, len(self._xyz), _p(self._xyz), len(self._el), _p(self._el),
                                    _p(self._np), int(nparts), ctypes.byref(self._h))
        if rc:
            raise RuntimeError("oracle layout failed with status %d" % rc)
        info = np.zeros(8, np.int64)
        lib().lso_layout_info(self._h, _p(info))
        self.info = dict(zip(["nparts", "full", "lep", "lvp", "lim", "nadj", "nv", "ne"], (int(x) for x in info)))

    def __del__(self):
        try:
            if self._h:
                lib().lso_layout_free(self._h)
        except Exception:
            pass

    def array(self, name):
        i = self.info
        d1 = self.dim + 1
        sizes = {
            "ele_permute": i["full"], "ele_offsets": i["nparts"] + 1, "vert_permute": i["nv"],
            "vert_ipermute": i["nv"], "vert_offsets": i["nparts"] + 1, "ele_after_permute": d1 * i["full"],
            "mem_locations": d1 * i["full"], "mem_location_offsets": i["nv"] + 1,
            "block_xadj": i["nparts"] + 1, "block_adjncy": i["nadj"],
            "local_coords": (6 if self.dim == 3 else 3) * i["full"],
        }
        out = np.zeros(sizes[name], np.float32 if name == "local_coords" else np.int32)
        rc = lib().lso_layout_copy(self._h, ARRAYS[name], _p(out))
        if rc:
            raise RuntimeError("oracle layout copy failed")
        return out

    def params(self, **kw):
        p = Params()
        p.dim = self.dim
        p.precision = 32
        for k, v in kw.items():
            setattr(p, k, v)
        return p

    def solve(self, params, phi0, vel, nsteps, nb_sets=True):
        nv, npt = self.info["nv"], self.info["nparts"]
        phi0 = np.ascontiguousarray(phi0, np.float32)
        velp = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        hist = np.zeros((nsteps + 1, nv), np.float32)
        nbs = np.zeros((max(nsteps, 1), npt), np.uint8) if nb_sets else None
        iters = np.zeros(max(nsteps, 1), np.int32)
        st = Stats()
        rc = lib().lso_solve(self._h, ctypes.byref(params), _p(phi0), _p(velp) if velp is not None else None,
                             nsteps, _p(hist), _p(nbs) if nbs is not None else None, _p(iters), ctypes.byref(st))
        s = st.as_dict()
        s["rc"] = rc
        n = st.steps_run
        return hist[: n + 1], (nbs[:n] if nbs is not None else None), iters[:n], s

    def update_only(self, params, phi, vel, nb_list):
        nv = self.info["nv"]
        phi = np.ascontiguousarray(phi, np.float32)
        velp = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        nb = np.ascontiguousarray(nb_list, np.int32)
        out = np.zeros(nv, np.float32)
        rc = lib().lso_update_only(self._h, ctypes.byref(params), _p(phi), _p(velp) if velp is not None else None,
                                   _p(nb), len(nb), _p(out))
        if rc:
            raise RuntimeError("oracle update failed %d" % rc)
        return out


UPDATE = {"advect": 0, "curvature": 1, "none": 2}
