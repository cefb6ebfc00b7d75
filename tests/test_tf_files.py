"""1D transfer-function files (.1dt, DemoData/c60.1dt) through the C ABI, host only."""
import ctypes as C

import numpy as np
import pytest

from imagevis3d_gb300 import _lib as L


def _write_1dt(path, tf):
    with open(path, "w") as f:
        f.write("%d\n" % len(tf))
        for r in tf:
            f.write("%s \n" % " ".join(repr(float(x)) for x in r))


def load(path, target=0, cap=65536):
    out = np.zeros((cap, 4), np.float32)
    n = C.c_int()
    L.call("gbvr_load_tf1d_file", path.encode(), target, out.ctypes.data_as(L.FP), cap, C.byref(n))
    return out[:n.value]


def test_c60_1dt_roundtrip(c60, tmp_path):
    p = str(tmp_path / "c60.1dt")
    _write_1dt(p, c60["tf1d"])
    tf = load(p)
    assert tf.shape == (256, 4) and np.array_equal(tf, c60["tf1d"])


def test_resampling_is_linear(tmp_path):
    p = str(tmp_path / "ramp.1dt")
    _write_1dt(p, np.array([[0, 0, 0, 0], [1, 0.5, 0.25, 1]], np.float32))
    tf = load(p, target=5)
    assert np.allclose(tf[:, 0], [0, 0.25, 0.5, 0.75, 1.0]) and np.allclose(tf[:, 3], tf[:, 0])
    assert load(p, target=2).shape == (2, 4)


def test_bad_files(tmp_path):
    p = str(tmp_path / "bad.1dt")
    open(p, "w").write("3\n1 2 3 4\n")
    with pytest.raises(L.GbvrError) as e:
        load(p)
    assert e.value.code == -5
    with pytest.raises(L.GbvrError) as e:
        load(str(tmp_path / "missing.1dt"))
    assert e.value.code == -4
