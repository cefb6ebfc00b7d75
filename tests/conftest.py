import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# Root of an ImageVis3D source tree (for the one test that reads the
# reference's own DemoData/c60.uvf); unset: that test is skipped.  The other
# parity tests use the fixtures under tests/golden/.
REFERENCE = os.environ.get("IMAGEVIS3D_REFERENCE", "")
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
    if not REFERENCE:
        pytest.skip("IMAGEVIS3D_REFERENCE (an ImageVis3D source tree) is not set")
    p = os.path.join(REFERENCE, rel)
    if not os.path.exists(p):
        pytest.skip("%s is not in the ImageVis3D tree at IMAGEVIS3D_REFERENCE" % rel)
    return p
