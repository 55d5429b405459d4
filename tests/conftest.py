import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def lib_built():
    """The CUDA library (host set-up entry points run without a GPU)."""
    from trans_bl_gb300 import api, build
    if not os.path.exists(api.LIB_PATH):
        build.build_library()
    return api.load()


@pytest.fixture(scope="session")
def oracle_built():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as ora
    ora.build()
    return ora
