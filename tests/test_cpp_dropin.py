"""The C++ LevelSet drop-in (include/LevelSet.h): a program written like the
reference's examples compiles and links against the library (CPU), and on
the GPU gives the same per-iteration results as the C ABI driven directly."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import lsgb300
import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "levelset_example.cpp")


def _compile(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "levelset_example")
    libdir = os.path.dirname(lsgb300.LIB_PATH)
    cmd = [cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe, "-L", libdir,
           "-llsgb300", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_example_compiles_and_links(tmp_path):
    exe = _compile(tmp_path)
    assert os.path.exists(exe)


def _read(path):
    raw = open(path, "rb").read()
    n, nv = np.frombuffer(raw[:8], np.int32)
    off = 8
    hist = np.frombuffer(raw[off:off + 4 * n * nv], np.float32).reshape(n, nv)
    off += 4 * n * nv
    ne = int(np.frombuffer(raw[off:off + 4], np.int32)[0])
    vel = np.frombuffer(raw[off + 4:off + 4 + 12 * ne], np.float32).reshape(ne, 3)
    return hist, vel


@pytest.mark.gpu
@pytest.mark.parametrize("tri", [False, True])
def test_dropin_equals_c_abi(tmp_path, tri):
    exe = _compile(tmp_path)
    if tri:
        xyz, el = synth.square_mesh(24, 0.2, seed=4)
        mesh = str(tmp_path / "sq.ply")
        synth.write_ply(mesh, xyz, [tuple(r) for r in el])
        h = 1.0 / 24
    else:
        xyz, el = synth.cube_mesh(10, 0.15, seed=4)
        mesh = str(tmp_path / "cube")
        synth.write_tetgen(mesh, xyz, el)
        h = 1.0 / 10
    nsteps, dt, bw, block = 4, 0.2 * h, 4 * h, 3
    out = str(tmp_path / "out.bin")
    r = subprocess.run([exe, mesh, "1" if tri else "0", str(nsteps), repr(dt), repr(bw), str(block), out],
                       capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    hist, vel = _read(out)
    assert hist.shape[0] == nsteps + 1
    for j in range(nsteps + 1):
        assert os.path.exists(str(tmp_path / ("result%d.vtk" % j)))
    assert open(str(tmp_path / "result.fld")).read().startswith("SCI\nASC\n2\n")

    p = lsgb300.default_params(num_steps=nsteps, time_step=dt, bandwidth=bw, block_size=block, partition_type=0)
    ls = lsgb300.LevelSet(tri, p)
    ls.load_mesh(mesh)
    ls.set_phi(hist[0])
    ls.set_velocity(vel)
    ls.setup()
    ref, done = ls.solve(nsteps)
    assert done == nsteps
    assert np.array_equal(hist.view(np.uint32), ref.view(np.uint32))
