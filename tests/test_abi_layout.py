"""The ctypes mirror (lsgb300.py) against the C header: every struct the
Python side declares has the size and field offsets the C compiler gives it
from include/lsgb300.h, so that a field added on one side only is caught on
the CPU (a C program compiled with the host compiler prints the layout)."""
import ctypes
import os
import shutil
import subprocess

import pytest

import lsgb300

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")

MIRRORS = [("ls_params", lsgb300.Params), ("ls_stats", lsgb300.Stats), ("ls_tune_trial", lsgb300.TuneTrial),
           ("ls_tune_report", lsgb300.TuneReport)]


def _c_layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "lsgb300.h"', "int main(void) {"]
    for cname, py in MIRRORS:
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c11", "-I", INCLUDE, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    layout = {}
    for line in out.splitlines():
        struct, field, value = line.split()
        layout[(struct, field)] = int(value)
    return layout


def test_ctypes_mirror_matches_c_header(tmp_path):
    layout = _c_layout(tmp_path)
    for cname, py in MIRRORS:
        assert ctypes.sizeof(py) == layout[(cname, "sizeof")], cname
        for fname, _ in py._fields_:
            assert getattr(py, fname).offset == layout[(cname, fname)], (cname, fname)
