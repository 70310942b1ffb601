import json
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


@pytest.fixture(scope="session")
def parity_report():
    """Returns record(name, **numbers): appends one JSON line per call to the
    file PTGPU_PARITY_REPORT names (nothing when it is unset), so a GPU run
    can keep the measured parity figures (RMSE, identical fractions)."""
    path = os.environ.get("PTGPU_PARITY_REPORT")

    def record(name, **numbers):
        line = dict(test=name, **{k: (float(v) if hasattr(v, "__float__") else v)
                                  for k, v in numbers.items()})
        print(json.dumps(line))
        if path:
            with open(path, "a") as f:
                f.write(json.dumps(line) + "\n")
    return record
