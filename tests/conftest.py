import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

REFERENCE = "/root/reference"
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the native kernels)")


@pytest.fixture(scope="session")
def c60():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "c60.npz")))


@pytest.fixture(scope="session")
def orc():
    from oracle import orc as o
    o.lib()
    return o


def reference_file(rel):
    p = os.path.join(REFERENCE, rel)
    if not os.path.exists(p):
        pytest.skip("reference tree not present (only in the build container)")
    return p
