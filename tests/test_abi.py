"""The C-ABI library loads without a GPU and exports every declared entry."""
import ctypes
import os
import re

import lsgb300

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:ls_status|const char\*|int|void)\s+(ls_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_loads_and_exports_all_symbols():
    lib = ctypes.CDLL(lsgb300.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(lsgb300.EXPORTS) <= names


def test_version_and_defaults():
    assert b"sm_103a" in lsgb300.lib().ls_version()
    p = lsgb300.default_params()
    # reference LevelSet defaults (LevelSet.cu:4-22)
    assert (p.num_steps, p.time_step, p.inside_iterations, p.block_size, p.side_lengths) == (10, 1.0, 1, 16, 1)
    assert (p.bandwidth, p.metis_size, p.partition_type) == (16.0, 16, 0)
