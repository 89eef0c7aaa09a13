"""Build oracle/_ref/: parts of the reference compiled from its own sources.

Recipe (test infrastructure only).  Compiles, with nvcc and the shim headers
in oracle/ref_shim/, directly from the reference tree (read-only):
  libref_tet.so  localSolverTet1Levelset  (src/core3d/include/redistance_kernels3d.h)
  libref_tri.so  localSolverTri, localSolverTet1 (src/core2d/include/redistance_kernels.h)
  libref_k20.so  meshFIM3d::updateT_single_stage from src/core3d/cuda/meshFIM3d.cu
                 (+ src/core3d/cuda/redistance3d.cu, which it links against)
  libref_layout3d.so, libref_layout2d.so
                 the patch layout (InitPatches, InitPatches2,
                 GenerateBlockNeighbors, GraphPartition_Square) from
                 src/core{3,2}d/cuda/meshFIM{3,2}d.cu, linked without the CUDA
                 runtime: oracle/ref_host_launch.cpp runs their kernels on the
                 CPU (oracle/ref_harness_layout{3,2}d.cu drive them); the 3D
                 library also runs the reference's whole time step
                 (meshFIM3d::GenerateData, oracle/ref_harness_layout3d.cu)
Nothing is copied into the repository; outputs go only to oracle/_ref/ (the
host build of the kernels reads copies of the kernel headers written there
with their dynamic shared-memory declaration pointed at a host buffer).

Usage: python oracle/build_ref.py [REFERENCE_ROOT]
REFERENCE_ROOT defaults to the LS_REFERENCE_ROOT environment variable, else
/root/reference; without a reference tree nothing is built.
Constants the reference takes from its missing dependency: LARGENUM = 1e9,
SMALLNUM = 1e-5 (the value src/core2d/include/redistance.h:17-19 uses).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "ref_shim")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in ("/usr/local/cuda/bin/nvcc", "nvcc"):
        if os.path.sep not in c or os.path.exists(c):
            return c
    return "nvcc"


def nvcc_path():
    import shutil

    c = nvcc()
    return c if os.path.sep in c else (shutil.which(c) or "/usr/local/cuda/bin/nvcc")


def run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


# the declaration of the kernels' dynamic shared memory, and what the host
# copies of the kernels (oracle/ref_host_launch.cpp) declare in its place
DYN_SMEM_DECL = "extern __shared__ char s_array[];"
DYN_SMEM_HOST = "char* s_array = dyn_smem;"
HOST_HEADERS = {3: ["meshFIM_kernels.h", "redistance_kernels3d.h"], 2: ["meshFIM2d_kernels.h"]}


def generate_host_headers(src):
    """Copies of the reference's kernel headers into oracle/_ref/gen{3,2}d/
    for the host build of the kernels, with one change: the dynamic
    shared-memory declaration becomes a pointer to the host buffer (a C++
    function cannot declare an extern array as a static).  Returns the
    include directory per dimension."""
    out = {}
    for d, names in HOST_HEADERS.items():
        gdir = os.path.join(OUT, "gen%dd" % d)
        os.makedirs(gdir, exist_ok=True)
        for name in names:
            text = open(os.path.join(src, "core%dd" % d, "include", name)).read()
            if DYN_SMEM_DECL not in text:
                raise RuntimeError("%s: dynamic shared-memory declaration not found" % name)
            with open(os.path.join(gdir, name), "w") as f:
                f.write(text.replace(DYN_SMEM_DECL, DYN_SMEM_HOST))
        out[d] = gdir
    return out


def default_root():
    return os.environ.get("LS_REFERENCE_ROOT", "/root/reference")


def build(ref_root=None):
    src = os.path.join(ref_root or default_root(), "src")
    if not os.path.isdir(src):
        return False
    os.makedirs(OUT, exist_ok=True)
    base = [nvcc(), "-std=c++17", "-O2", "-Xcompiler", "-fPIC,-ffp-contract=off", "-w"] + ARCH + [
        "-I" + SHIM, "-include", os.path.join(SHIM, "prelude.h"), "-DSMALLNUM=1e-5"]
    inc3 = ["-I" + os.path.join(src, "core3d", "include")]
    inc2 = ["-I" + os.path.join(src, "core2d", "include")]
    jobs = [
        (base + inc3 + ["-c", os.path.join(HERE, "ref_harness_tet.cu"), "-o", os.path.join(OUT, "tet.o")]),
        (base + inc2 + ["-c", os.path.join(HERE, "ref_harness_tri.cu"), "-o", os.path.join(OUT, "tri.o")]),
        (base + inc3 + ["-DLSREF_HOST_ONLY", "-c", os.path.join(src, "core3d", "cuda", "meshFIM3d.cu"),
                        "-o", os.path.join(OUT, "meshFIM3d.o")]),
        (base + inc3 + ["-DLSREF_HOST_ONLY", "-c", os.path.join(src, "core3d", "cuda", "redistance3d.cu"),
                        "-o", os.path.join(OUT, "redistance3d.o")]),
        (base + inc3 + ["-DLSREF_HOST_ONLY", "-c", os.path.join(HERE, "ref_harness_k20.cu"),
                        "-o", os.path.join(OUT, "k20.o")]),
    ]
    o = lambda n: os.path.join(OUT, n)  # noqa: E731
    host = ["-DLSREF_HOST_ONLY", "-c"]
    jobs += [
        (base + inc3 + host + [os.path.join(HERE, "ref_harness_layout3d.cu"), "-o", o("layout3d.o")]),
        (base + inc2 + host + [os.path.join(HERE, "ref_harness_layout2d.cu"), "-o", o("layout2d.o")]),
        (base + inc2 + host + [os.path.join(src, "core2d", "cuda", "meshFIM2d.cu"), "-o", o("meshFIM2d.o")]),
        (base + inc2 + host + [os.path.join(src, "core2d", "cuda", "redistance.cu"), "-o", o("redistance2d.o")]),
    ]
    # the kernel-launch stand-ins, with the host compiler, on the kernel
    # headers as generate_host_headers leaves them
    gen = generate_host_headers(src)
    gxx = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-w", "-DSMALLNUM=1e-5", "-I" + SHIM,
           "-I" + os.path.join(os.path.dirname(os.path.dirname(nvcc_path())), "include")]
    for d, inc in ((3, inc3), (2, inc2)):
        jobs.append(gxx + ["-I" + gen[d]] + inc + ["-DLSREF_DIM=%d" % d, "-c",
                                                   os.path.join(HERE, "ref_host_launch.cpp"),
                                                   "-o", o("host_launch%dd.o" % d)])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, jobs))
    link = [nvcc(), "-shared"] + ARCH
    run(link + [o("tet.o"), "-o", o("libref_tet.so")])
    run(link + [o("tri.o"), "-o", o("libref_tri.so")])
    run(link + [o(n) for n in ("k20.o", "meshFIM3d.o", "redistance3d.o")] + ["-o", o("libref_k20.so")])
    # no CUDA runtime: every launch goes to the host stand-ins
    run(["g++", "-shared", "-Wl,--no-undefined", "-o", o("libref_layout3d.so")] +
        [o(n) for n in ("layout3d.o", "meshFIM3d.o", "redistance3d.o", "host_launch3d.o")])
    run(["g++", "-shared", "-Wl,--no-undefined", "-o", o("libref_layout2d.so")] +
        [o(n) for n in ("layout2d.o", "meshFIM2d.o", "redistance2d.o", "host_launch2d.o")])
    return True


if __name__ == "__main__":
    ok = build(sys.argv[1] if len(sys.argv) > 1 else None)
    print("built" if ok else "reference tree not found; nothing built")
