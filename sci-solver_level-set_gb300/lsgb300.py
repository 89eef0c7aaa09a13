"""ctypes binding of the lsgb300 C ABI (include/lsgb300.h).

The binding is a thin host-side mirror of the reference's LevelSet call
sequence (src/LevelSet.cu): create, set the mesh, phi and per-element
velocity, solve, read results.  All compute runs in liblsgb300.so (CUDA,
sm_103a); loading fails loudly if the library has not been built.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblsgb300.so")

LS_OK, LS_BAD_INPUT, LS_PATCH_TOO_LARGE, LS_DEVICE_TIMEOUT, LS_CUDA_ERROR, LS_NOT_READY, LS_NO_MEMORY = range(7)
UPDATE_ADVECT, UPDATE_CURVATURE, UPDATE_NONE = 0, 1, 2
REF_COMPAT, FP64_FLAGGED, PROFILE, NO_GRAPH, BITEXACT = 1, 2, 4, 8, 16
HOST_STAGING = 1 << 5
PERSISTENT = 1 << 6

# reference-format layout arrays (ls_get_layout selectors)
REF_ARRAYS = {
    "ele_permute": 0, "ele_offsets": 1, "vert_permute": 2, "vert_offsets": 3,
    "ele_after_permute": 4, "mem_locations": 5, "mem_location_offsets": 6,
    "block_xadj": 7, "block_adjncy": 8, "local_coords": 9, "vert_ipermute": 10,
}


class Params(ctypes.Structure):
    _fields_ = [
        ("num_steps", ctypes.c_int), ("time_step", ctypes.c_double), ("inside_iterations", ctypes.c_int),
        ("block_size", ctypes.c_int), ("side_lengths", ctypes.c_int), ("bandwidth", ctypes.c_double),
        ("metis_size", ctypes.c_int), ("partition_type", ctypes.c_int), ("verbose", ctypes.c_int),
        ("update_kind", ctypes.c_int), ("curv_coeff", ctypes.c_double), ("flags", ctypes.c_uint),
        ("fim_sweeps", ctypes.c_int), ("max_fim_iters", ctypes.c_int), ("smallnum", ctypes.c_double),
        ("largenum", ctypes.c_double), ("length_scale", ctypes.c_double), ("fp64_threshold", ctypes.c_double),
        ("graph_chunk", ctypes.c_int), ("fim_ctas_per_sm", ctypes.c_int), ("barrier_wait_limit", ctypes.c_int),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("steps_run", ctypes.c_int), ("fim_iters", ctypes.c_longlong), ("patch_visits", ctypes.c_longlong),
        ("check_visits", ctypes.c_longlong), ("nb_vertex_updates", ctypes.c_longlong),
        ("nb_patch_vertices", ctypes.c_longlong), ("nb_patches", ctypes.c_longlong),
        ("flagged_copies", ctypes.c_longlong), ("ms_total", ctypes.c_double),
        ("ms_sweep", ctypes.c_double), ("ms_check", ctypes.c_double), ("ms_schedule", ctypes.c_double),
        ("ms_seed", ctypes.c_double), ("ms_narrowband", ctypes.c_double), ("ms_update", ctypes.c_double),
        ("n_sweep", ctypes.c_longlong), ("n_check", ctypes.c_longlong), ("n_schedule", ctypes.c_longlong),
        ("n_seed", ctypes.c_longlong), ("n_narrowband", ctypes.c_longlong), ("n_update", ctypes.c_longlong),
        ("sweep_slab_bytes", ctypes.c_longlong), ("kernel_launches", ctypes.c_longlong),
        ("warm_vertices", ctypes.c_longlong), ("unsupported_resets", ctypes.c_longlong),
        ("support_rounds", ctypes.c_longlong), ("moved_vertices", ctypes.c_longlong),
        ("learned_fallbacks", ctypes.c_longlong), ("pairs_collected", ctypes.c_longlong),
        ("early_visits", ctypes.c_longlong),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# every entry point declared in include/lsgb300.h
EXPORTS = [
    "ls_default_params", "ls_create", "ls_destroy", "ls_set_params", "ls_get_params", "ls_set_mesh",
    "ls_set_partition", "ls_set_phi", "ls_set_velocity", "ls_prepare", "ls_setup", "ls_solve", "ls_step",
    "ls_step_host", "ls_get_phi", "ls_get_stats", "ls_reset_stats", "ls_get_launch_log", "ls_get_narrowband",
    "ls_get_layout_info", "ls_get_layout", "ls_last_error", "ls_version", "ls_partition_structured",
    "ls_partition_rcb", "ls_set_profile", "ls_debug_active", "ls_narrowband_noalloc", "ls_load_mesh",
    "ls_get_mesh_info", "ls_get_mesh", "ls_write_vtk", "ls_eikonal", "ls_batch_create", "ls_batch_destroy",
    "ls_batch_last_error", "ls_batch_add", "ls_batch_setup", "ls_batch_solve", "ls_batch_get_phi",
    "ls_batch_get_stats", "ls_batch_reset_stats", "ls_batch_set_profile", "ls_batch_get_layout_info",
    "ls_batch_get_layout", "ls_autotune", "ls_mlp_create", "ls_mlp_destroy", "ls_mlp_last_error",
    "ls_mlp_num_params", "ls_mlp_set_params", "ls_mlp_get_params", "ls_mlp_predict", "ls_mlp_gradients",
    "ls_mlp_train", "ls_mlp_reserve_pairs", "ls_mlp_clear_pairs", "ls_mlp_num_pairs", "ls_mlp_train_pairs",
    "ls_learn_collect", "ls_set_learned", "ls_batch_set_learned", "ls_mlp_eval_pairs", "ls_batch_autotune",
    "ls_partition_graph", "ls_edge_cut",
]

class TuneTrial(ctypes.Structure):
    _fields_ = [("patch_size", ctypes.c_int), ("fim_ctas_per_sm", ctypes.c_int), ("ms_per_step", ctypes.c_double),
                ("updates_per_s", ctypes.c_double)]


class TuneReport(ctypes.Structure):
    _fields_ = [("ntrials", ctypes.c_int), ("best", ctypes.c_int), ("trials", TuneTrial * 32)]


_lib = None


def lib():
    """Load liblsgb300.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("liblsgb300.so not built; run __graft_entry__.build() first (%s)" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    P, I, F, V = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_void_p
    L.ls_default_params.argtypes = [ctypes.POINTER(Params)]
    L.ls_create.argtypes = [ctypes.POINTER(P), I]
    L.ls_destroy.argtypes = [P]
    L.ls_set_params.argtypes = [P, ctypes.POINTER(Params)]
    L.ls_get_params.argtypes = [P, ctypes.POINTER(Params)]
    L.ls_set_mesh.argtypes = [P, V, I, V, I]
    L.ls_set_partition.argtypes = [P, V, I]
    L.ls_set_phi.argtypes = [P, V]
    L.ls_set_velocity.argtypes = [P, V]
    L.ls_prepare.argtypes = [P]
    L.ls_setup.argtypes = [P]
    L.ls_solve.argtypes = [P, I, V, ctypes.POINTER(I)]
    L.ls_step.argtypes = [P, I, ctypes.POINTER(I)]
    L.ls_step_host.argtypes = [P, V, V]
    L.ls_get_phi.argtypes = [P, V]
    L.ls_get_stats.argtypes = [P, ctypes.POINTER(Stats)]
    L.ls_reset_stats.argtypes = [P]
    L.ls_get_launch_log.argtypes = [P, I, V, V, V, ctypes.POINTER(I)]
    L.ls_set_profile.argtypes = [P, I]
    L.ls_debug_active.argtypes = [P, V, I, ctypes.POINTER(I), V]
    L.ls_load_mesh.argtypes = [P, ctypes.c_char_p]
    L.ls_get_mesh_info.argtypes = [P, ctypes.POINTER(I), ctypes.POINTER(I)]
    L.ls_get_mesh.argtypes = [P, V, V]
    L.ls_write_vtk.argtypes = [P, ctypes.c_char_p, V]
    L.ls_eikonal.argtypes = [P, V, V, I, V]
    L.ls_autotune.argtypes = [P, I, ctypes.POINTER(TuneReport)]
    L.ls_mlp_create.argtypes = [ctypes.POINTER(P), ctypes.c_ulonglong]
    L.ls_mlp_destroy.argtypes = [P]
    L.ls_mlp_last_error.argtypes = [P]
    L.ls_mlp_last_error.restype = ctypes.c_char_p
    L.ls_mlp_num_params.argtypes = []
    L.ls_mlp_set_params.argtypes = [P, V]
    L.ls_mlp_get_params.argtypes = [P, V]
    L.ls_mlp_predict.argtypes = [P, V, I, V]
    L.ls_mlp_gradients.argtypes = [P, V, V, I, V, ctypes.POINTER(ctypes.c_float)]
    L.ls_mlp_train.argtypes = [P, V, V, I, I, I, ctypes.c_float, ctypes.POINTER(ctypes.c_float)]
    L.ls_mlp_reserve_pairs.argtypes = [P, ctypes.c_longlong]
    L.ls_mlp_clear_pairs.argtypes = [P]
    L.ls_mlp_num_pairs.argtypes = [P, ctypes.POINTER(ctypes.c_longlong)]
    L.ls_mlp_train_pairs.argtypes = [P, I, I, ctypes.c_float, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_float)]
    L.ls_learn_collect.argtypes = [P, P, I, ctypes.POINTER(I)]
    L.ls_set_learned.argtypes = [P, P, ctypes.c_double, ctypes.c_double, I]
    L.ls_batch_set_learned.argtypes = [P, P, ctypes.c_double, ctypes.c_double, I]
    L.ls_batch_autotune.argtypes = [P, I, V]
    L.ls_mlp_eval_pairs.argtypes = [P, ctypes.c_longlong, ctypes.c_longlong, V]
    L.ls_batch_create.argtypes = [ctypes.POINTER(P)]
    L.ls_batch_destroy.argtypes = [P]
    L.ls_batch_last_error.argtypes = [P]
    L.ls_batch_last_error.restype = ctypes.c_char_p
    L.ls_batch_add.argtypes = [P, P, ctypes.POINTER(I)]
    L.ls_batch_setup.argtypes = [P]
    L.ls_batch_solve.argtypes = [P, I, ctypes.POINTER(I)]
    L.ls_batch_get_phi.argtypes = [P, I, V]
    L.ls_batch_get_stats.argtypes = [P, ctypes.POINTER(Stats)]
    L.ls_batch_reset_stats.argtypes = [P]
    L.ls_batch_set_profile.argtypes = [P, I]
    L.ls_batch_get_layout_info.argtypes = [P, V]
    L.ls_batch_get_layout.argtypes = [P, I, V]
    L.ls_narrowband_noalloc.argtypes = [I, I, V, V, V, ctypes.c_float, ctypes.c_float, ctypes.c_float, V, V, V, V]
    L.ls_get_narrowband.argtypes = [P, V]
    L.ls_get_layout_info.argtypes = [P, V]
    L.ls_get_layout.argtypes = [P, I, V]
    L.ls_last_error.argtypes = [P]
    L.ls_last_error.restype = ctypes.c_char_p
    L.ls_version.restype = ctypes.c_char_p
    L.ls_partition_structured.argtypes = [I, I, I, I, V, ctypes.POINTER(I)]
    L.ls_partition_rcb.argtypes = [I, V, I, I, V, ctypes.POINTER(I)]
    L.ls_partition_graph.argtypes = [I, V, I, I, I, V, ctypes.POINTER(I)]
    L.ls_edge_cut.argtypes = [I, V, I, I, V, ctypes.POINTER(ctypes.c_longlong)]
    for name in EXPORTS:
        fn = getattr(L, name)
        if name not in ("ls_last_error", "ls_version", "ls_batch_last_error", "ls_mlp_last_error"):
            fn.restype = ctypes.c_int
    _lib = L
    return L


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class LevelSetError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("ls status %d: %s" % (code, msg))
        self.code = code


def default_params(**kw):
    p = Params()
    lib().ls_default_params(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def partition_structured(dim, nside, block, nv):
    npart = np.zeros(nv, np.int32)
    n = ctypes.c_int(0)
    rc = lib().ls_partition_structured(dim, nside, block, nv, _ptr(npart), ctypes.byref(n))
    if rc:
        raise LevelSetError(rc, "structured partition")
    return npart, n.value


def partition_rcb(dim, xyz, target):
    xyz = np.ascontiguousarray(xyz, np.float32)
    npart = np.zeros(len(xyz), np.int32)
    n = ctypes.c_int(0)
    rc = lib().ls_partition_rcb(dim, _ptr(xyz), len(xyz), target, _ptr(npart), ctypes.byref(n))
    if rc:
        raise LevelSetError(rc, "rcb partition")
    return npart, n.value


def partition_graph(dim, elems, nv, target):
    el = np.ascontiguousarray(elems, np.int32)
    npart = np.zeros(nv, np.int32)
    n = ctypes.c_int(0)
    rc = lib().ls_partition_graph(dim, _ptr(el), len(el), nv, target, _ptr(npart), ctypes.byref(n))
    if rc:
        raise LevelSetError(rc, "graph partition")
    return npart, n.value


def edge_cut(dim, elems, nv, npart):
    el = np.ascontiguousarray(elems, np.int32)
    a = np.ascontiguousarray(npart, np.int32)
    cut = ctypes.c_longlong(0)
    rc = lib().ls_edge_cut(dim, _ptr(el), len(el), nv, _ptr(a), ctypes.byref(cut))
    if rc:
        raise LevelSetError(rc, "edge cut")
    return cut.value


class LevelSet:
    """Handle over the C ABI.  Same life cycle as the reference LevelSet."""

    def __init__(self, is_tri, params=None):
        self._h = ctypes.c_void_p()
        rc = lib().ls_create(ctypes.byref(self._h), 1 if is_tri else 0)
        if rc:
            raise LevelSetError(rc, "create")
        self.is_tri = bool(is_tri)
        self.nv = 0
        self.ne = 0
        if params is not None:
            self.set_params(params)

    def close(self):
        if self._h:
            lib().ls_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != LS_OK:
            raise LevelSetError(rc, "%s: %s" % (what, lib().ls_last_error(self._h).decode()))

    def set_params(self, p):
        self._check(lib().ls_set_params(self._h, ctypes.byref(p)), "set_params")

    def set_mesh(self, xyz, elems):
        self._xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
        self._elems = np.ascontiguousarray(elems, np.int32)
        self.nv, self.ne = len(self._xyz), len(self._elems)
        self._check(lib().ls_set_mesh(self._h, _ptr(self._xyz), self.nv, _ptr(self._elems), self.ne), "set_mesh")

    def load_mesh(self, filename):
        self._check(lib().ls_load_mesh(self._h, filename.encode()), "load_mesh")
        nv, ne = ctypes.c_int(0), ctypes.c_int(0)
        lib().ls_get_mesh_info(self._h, ctypes.byref(nv), ctypes.byref(ne))
        self.nv, self.ne = nv.value, ne.value
        self._xyz = np.zeros((self.nv, 3), np.float32)
        self._elems = np.zeros((self.ne, 3 if self.is_tri else 4), np.int32)
        lib().ls_get_mesh(self._h, _ptr(self._xyz), _ptr(self._elems))
        return self._xyz, self._elems

    def write_vtk(self, path, phi):
        a = np.ascontiguousarray(phi, np.float32)
        self._check(lib().ls_write_vtk(self._h, path.encode(), _ptr(a)), "write_vtk")

    def eikonal(self, seeds, values):
        s = np.ascontiguousarray(seeds, np.int32)
        v = np.ascontiguousarray(values, np.float32)
        out = np.zeros(self.nv, np.float32)
        self._check(lib().ls_eikonal(self._h, _ptr(s), _ptr(v), len(s), _ptr(out)), "eikonal")
        return out

    def autotune(self, trial_steps=2):
        """ls_autotune: returns (trials, best index); the handle is left set up
        with the best patch size and CTAs per SM."""
        r = TuneReport()
        self._check(lib().ls_autotune(self._h, int(trial_steps), ctypes.byref(r)), "autotune")
        trials = [dict(patch_size=t.patch_size, fim_ctas_per_sm=t.fim_ctas_per_sm, ms_per_step=t.ms_per_step,
                       updates_per_s=t.updates_per_s) for t in r.trials[: r.ntrials]]
        return trials, r.best

    def get_params(self):
        p = Params()
        self._check(lib().ls_get_params(self._h, ctypes.byref(p)), "get_params")
        return p

    def learn_collect(self, mlp, nsteps):
        """ls_learn_collect: nsteps steps recording training pairs into mlp."""
        done = ctypes.c_int(0)
        self._check(lib().ls_learn_collect(self._h, mlp._m, int(nsteps), ctypes.byref(done)), "learn_collect")
        return done.value

    def set_learned(self, mlp, margin=0.0, support_tol=0.0, reset_mode=0):
        self._check(lib().ls_set_learned(self._h, mlp._m if mlp is not None else None, float(margin),
                                         float(support_tol), int(reset_mode)), "set_learned")

    def set_partition(self, npart, nparts):
        a = np.ascontiguousarray(npart, np.int32)
        self._check(lib().ls_set_partition(self._h, _ptr(a), int(nparts)), "set_partition")

    def set_phi(self, phi):
        a = np.ascontiguousarray(phi, np.float32)
        if self.nv and a.size != self.nv:
            raise LevelSetError(LS_BAD_INPUT, "Initialize values size does not match number of vertices!")
        self._check(lib().ls_set_phi(self._h, _ptr(a)), "set_phi")

    def set_velocity(self, vel):
        a = np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        if self.ne and len(a) != self.ne:
            raise LevelSetError(LS_BAD_INPUT, "Initialize values size does not match number of elements!")
        self._check(lib().ls_set_velocity(self._h, _ptr(a)), "set_velocity")

    def prepare(self):
        self._check(lib().ls_prepare(self._h), "prepare")

    def setup(self):
        self._check(lib().ls_setup(self._h), "setup")

    def solve(self, nsteps, history=True):
        hist = np.zeros((nsteps + 1, self.nv), np.float32) if history else None
        done = ctypes.c_int(0)
        self._check(lib().ls_solve(self._h, nsteps, _ptr(hist) if hist is not None else None, ctypes.byref(done)),
                    "solve")
        return (hist[: done.value + 1] if hist is not None else None), done.value

    def step(self, nsteps=1):
        done = ctypes.c_int(0)
        self._check(lib().ls_step(self._h, nsteps, ctypes.byref(done)), "step")
        return done.value

    def step_host(self, phi_in, phi_out):
        self._check(lib().ls_step_host(self._h, _ptr(phi_in), _ptr(phi_out)), "step_host")

    def phi(self):
        out = np.zeros(self.nv, np.float32)
        self._check(lib().ls_get_phi(self._h, _ptr(out)), "get_phi")
        return out

    def stats(self):
        s = Stats()
        self._check(lib().ls_get_stats(self._h, ctypes.byref(s)), "get_stats")
        return s.as_dict()

    def set_profile(self, on):
        self._check(lib().ls_set_profile(self._h, 1 if on else 0), "set_profile")

    def reset_stats(self):
        self._check(lib().ls_reset_stats(self._h), "reset_stats")

    def launch_log(self):
        """FIM kernel launches of the profiled steps since the last
        reset_stats: (kinds [0 sweep, 1 check], device ms, algorithmic slab
        bytes) as numpy arrays."""
        n = ctypes.c_int(0)
        self._check(lib().ls_get_launch_log(self._h, 0, None, None, None, ctypes.byref(n)), "get_launch_log")
        k = n.value
        kinds = np.zeros(k, np.int32)
        ms = np.zeros(k, np.float64)
        nbytes = np.zeros(k, np.int64)
        if k:
            self._check(lib().ls_get_launch_log(self._h, k, _ptr(kinds), _ptr(ms), _ptr(nbytes), ctypes.byref(n)),
                        "get_launch_log")
        return kinds, ms, nbytes

    def narrowband(self, nparts):
        out = np.zeros(nparts, np.uint8)
        self._check(lib().ls_get_narrowband(self._h, _ptr(out)), "get_narrowband")
        return out

    def debug_active(self, with_dt=False):
        cap = 1 << 20
        lst = np.zeros(cap, np.int32)
        n = ctypes.c_int(0)
        dt = np.zeros(self.nv, np.float32) if with_dt else None
        self._check(lib().ls_debug_active(self._h, _ptr(lst), cap, ctypes.byref(n),
                                          _ptr(dt) if dt is not None else None), "debug_active")
        return lst[: n.value].copy(), dt

    def layout_info(self):
        info = np.zeros(10, np.int64)
        self._check(lib().ls_get_layout_info(self._h, _ptr(info)), "layout_info")
        keys = ["nparts", "full", "lep", "lvp", "lgp", "lim", "nadj", "nv", "ne", "dim"]
        return dict(zip(keys, (int(x) for x in info)))

    def layout(self, name):
        out = _layout_buffer(self.layout_info(), name)
        self._check(lib().ls_get_layout(self._h, REF_ARRAYS[name], _ptr(out)), "layout")
        return out


_LAYOUT_KEYS = ["nparts", "full", "lep", "lvp", "lgp", "lim", "nadj", "nv", "ne", "dim"]


def _layout_buffer(info, name):
    d1 = info["dim"] + 1
    sizes = {
        "ele_permute": info["full"], "ele_offsets": info["nparts"] + 1, "vert_permute": info["nv"],
        "vert_ipermute": info["nv"], "vert_offsets": info["nparts"] + 1,
        "ele_after_permute": d1 * info["full"], "mem_locations": d1 * info["full"],
        "mem_location_offsets": info["nv"] + 1, "block_xadj": info["nparts"] + 1,
        "block_adjncy": info["nadj"], "local_coords": (6 if d1 == 4 else 3) * info["full"],
    }
    return np.zeros(sizes[name], np.float32 if name == "local_coords" else np.int32)


class LevelSetBatch:
    """Batch of independent meshes stepped together (ls_batch_*)."""

    def __init__(self):
        self._b = ctypes.c_void_p()
        rc = lib().ls_batch_create(ctypes.byref(self._b))
        if rc:
            raise LevelSetError(rc, "batch create")
        self.sizes = []

    def close(self):
        if self._b:
            lib().ls_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != LS_OK:
            raise LevelSetError(rc, "%s: %s" % (what, lib().ls_batch_last_error(self._b).decode()))

    def add(self, ls):
        idx = ctypes.c_int(-1)
        self._check(lib().ls_batch_add(self._b, ls._h, ctypes.byref(idx)), "batch add")
        self.sizes.append(ls.nv)
        return idx.value

    def setup(self):
        self._check(lib().ls_batch_setup(self._b), "batch setup")

    def solve(self, nsteps):
        done = ctypes.c_int(0)
        self._check(lib().ls_batch_solve(self._b, nsteps, ctypes.byref(done)), "batch solve")
        return done.value

    def phi(self, index):
        out = np.zeros(self.sizes[index], np.float32)
        self._check(lib().ls_batch_get_phi(self._b, index, _ptr(out)), "batch get_phi")
        return out

    def stats(self):
        s = Stats()
        self._check(lib().ls_batch_get_stats(self._b, ctypes.byref(s)), "batch stats")
        return s.as_dict()

    def reset_stats(self):
        self._check(lib().ls_batch_reset_stats(self._b), "batch reset_stats")

    def set_profile(self, on):
        self._check(lib().ls_batch_set_profile(self._b, 1 if on else 0), "batch set_profile")

    def autotune(self, trial_steps=2):
        """ls_batch_autotune: returns (trials, best index); the batch is left
        set up with the best patch size and FIM setting."""
        r = TuneReport()
        self._check(lib().ls_batch_autotune(self._b, int(trial_steps), ctypes.byref(r)), "batch autotune")
        trials = [dict(patch_size=t.patch_size, fim_ctas_per_sm=t.fim_ctas_per_sm, ms_per_step=t.ms_per_step,
                       updates_per_s=t.updates_per_s) for t in r.trials[: r.ntrials]]
        return trials, r.best

    def set_learned(self, mlp, margin=0.0, support_tol=0.0, reset_mode=0):
        self._check(lib().ls_batch_set_learned(self._b, mlp._m if mlp is not None else None, float(margin),
                                               float(support_tol), int(reset_mode)), "batch set_learned")

    def layout_info(self):
        info = np.zeros(10, np.int64)
        self._check(lib().ls_batch_get_layout_info(self._b, _ptr(info)), "batch layout_info")
        return dict(zip(_LAYOUT_KEYS, (int(x) for x in info)))

    def layout(self, name):
        out = _layout_buffer(self.layout_info(), name)
        self._check(lib().ls_batch_get_layout(self._b, REF_ARRAYS[name], _ptr(out)), "batch layout")
        return out


def from_workload(w, ref_compat=False, fp64_flagged=False, profile=False, setup=True, bit_exact=False, flags=0,
                  structured_block=0, **extra):
    """LevelSet handle for a synth.workload() dictionary (mesh, partition,
    phi0, velocity and the step parameters).  structured_block > 0: the
    library's structured partitioner with that block side on the lattice of
    w["n"] + 1 vertices per side, instead of the workload's partition."""
    flags = flags | ((REF_COMPAT if ref_compat else 0) | (FP64_FLAGGED if fp64_flagged else 0) | (PROFILE if profile else 0)
             | (BITEXACT if bit_exact else 0))
    kind = {"advect": UPDATE_ADVECT, "curvature": UPDATE_CURVATURE, "none": UPDATE_NONE}[w["update"]]
    if structured_block > 0:
        extra = dict(extra, partition_type=1, side_lengths=w["n"] + 1, block_size=structured_block)
    p = default_params(num_steps=w["steps"], time_step=w["dt"], bandwidth=w["bandwidth"], update_kind=kind,
                       curv_coeff=1.0, flags=flags, **extra)
    ls = LevelSet(w["dim"] == 2, p)
    ls.set_mesh(w["xyz"], w["elems"])
    if structured_block <= 0:
        ls.set_partition(w["npart"], w["nparts"])
    ls.set_phi(w["phi0"])
    ls.set_velocity(w["vel"])
    if setup:
        ls.setup()
    return ls


class MLP:
    """The learned warm start's network (ls_mlp_*)."""

    def __init__(self, seed=0):
        self._m = ctypes.c_void_p()
        rc = lib().ls_mlp_create(ctypes.byref(self._m), int(seed))
        if rc:
            raise LevelSetError(rc, "mlp create")
        self.nparams = lib().ls_mlp_num_params()

    def close(self):
        if self._m:
            lib().ls_mlp_destroy(self._m)
            self._m = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != LS_OK:
            raise LevelSetError(rc, "%s: %s" % (what, lib().ls_mlp_last_error(self._m).decode()))

    def set_params(self, p):
        a = np.ascontiguousarray(p, np.float32)
        assert a.size == self.nparams
        self._check(lib().ls_mlp_set_params(self._m, _ptr(a)), "mlp set_params")

    def params(self):
        out = np.zeros(self.nparams, np.float32)
        self._check(lib().ls_mlp_get_params(self._m, _ptr(out)), "mlp get_params")
        return out

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 128)
        y = np.zeros(len(x), np.float32)
        self._check(lib().ls_mlp_predict(self._m, _ptr(x), len(x), _ptr(y)), "mlp predict")
        return y

    def gradients(self, x, t):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 128)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(self.nparams, np.float32)
        loss = ctypes.c_float(0)
        self._check(lib().ls_mlp_gradients(self._m, _ptr(x), _ptr(t), len(x), _ptr(g), ctypes.byref(loss)),
                    "mlp gradients")
        return g, loss.value

    def reserve_pairs(self, capacity):
        self._check(lib().ls_mlp_reserve_pairs(self._m, int(capacity)), "mlp reserve_pairs")

    def clear_pairs(self):
        self._check(lib().ls_mlp_clear_pairs(self._m), "mlp clear_pairs")

    def num_pairs(self):
        n = ctypes.c_longlong(0)
        self._check(lib().ls_mlp_num_pairs(self._m, ctypes.byref(n)), "mlp num_pairs")
        return n.value

    def eval_pairs(self, first, count):
        """|prediction - target| / h of the pairs [first, first + count)."""
        out = np.zeros(int(count), np.float32)
        self._check(lib().ls_mlp_eval_pairs(self._m, int(first), int(count), _ptr(out)), "mlp eval_pairs")
        return out

    def train_pairs(self, epochs=1, batch=65536, lr=1e-3, seed=0):
        loss = ctypes.c_float(0)
        self._check(lib().ls_mlp_train_pairs(self._m, int(epochs), int(batch), float(lr), int(seed),
                                             ctypes.byref(loss)), "mlp train_pairs")
        return loss.value

    def train(self, x, t, epochs=1, batch=65536, lr=1e-3):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 128)
        t = np.ascontiguousarray(t, np.float32)
        loss = ctypes.c_float(0)
        self._check(lib().ls_mlp_train(self._m, _ptr(x), _ptr(t), len(x), int(epochs), int(batch), float(lr),
                                       ctypes.byref(loss)), "mlp train")
        return loss.value
