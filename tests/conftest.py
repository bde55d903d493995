import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def P():
    """The product package with its library built."""
    from plant_gb300 import buildlib as B
    B.build()
    import plant_gb300
    plant_gb300.lib()
    return plant_gb300


@pytest.fixture(scope="session")
def O():
    """The CPU oracle (test infrastructure)."""
    from oracle import oracle
    oracle.lib()
    return oracle


def label_case(name):
    base = os.path.join(GOLDEN, "labels", name)
    return {k: base + "." + k for k in ("gr", "order", "labels", "pairs", "dist")}
