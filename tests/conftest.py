import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def built_lib():
    """Builds (if needed) and loads libptgpu.so."""
    from ptgpu_pc_gb300 import build
    build.build()
    import ptgpu_pc_gb300
    return ptgpu_pc_gb300.lib()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle
