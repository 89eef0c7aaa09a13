"""Build liblsgb300.so (the CUDA sm_103a product library) in-tree.

    python sci-solver_level-set_gb300/build.py

Compiles every translation unit in csrc/ with nvcc for sm_103a only, in
parallel, and links one shared library with the CUDA runtime linked
statically.  Output: sci-solver_level-set_gb300/_build/liblsgb300.so.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liblsgb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["ls_layout.cpp", "ls_meshio.cpp", "ls_partition.cpp", "ls_api.cpp", "LevelSet.cpp", "ls_solver.cu", "ls_kernels.cu", "ls_kernels_exact.cu", "ls_noalloc.cu", "ls_mlp.cu"]
# translation units compiled without FMA contraction
NO_FMA = {"ls_kernels_exact.cu"}
# the fast kernel build: hardware-approximate division and square root
# (denormals kept); the bit-exact build keeps IEEE-rounded operations
FAST_DIV_SQRT = {"ls_kernels.cu"}


def nvcc():
    p = "/usr/local/cuda/bin/nvcc"
    return p if os.path.exists(p) else "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    # host code without FP contraction: the host-side local coordinates must
    # round exactly like the CPU oracle's on x86 and Arm alike
    flags = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
             "-I" + os.path.join(HERE, "..", "include")] + ARCH
    if ptxas_info:
        flags += ["-Xptxas", "-v"]
    jobs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        extra = ["-fmad=false"] if src in NO_FMA else []
        if src in FAST_DIV_SQRT:
            extra += ["-prec-div=false", "-prec-sqrt=false"]
        jobs.append([nvcc()] + flags + extra + ["-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(_run, jobs))
    _run([nvcc(), "-shared"] + ARCH + objs + ["-o", LIB])
    if verbose:
        for lg in logs:
            sys.stdout.write(lg)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="-v" in sys.argv))
