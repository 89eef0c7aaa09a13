import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "sci-solver_level-set_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the product library and the oracle once if they are missing."""
    import lsgb300
    import lsoracle

    if not os.path.exists(lsgb300.LIB_PATH):
        import build as pkg_build

        pkg_build.build()
    if not os.path.exists(lsoracle.LIB_PATH):
        lsoracle.build()
    yield
