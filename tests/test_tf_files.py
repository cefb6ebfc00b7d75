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


# ---- 2D transfer functions (.2dt, DemoData/c60.2dt) -------------------------

def _c60_2dt(c60, tmp_path):
    p = str(tmp_path / "c60.2dt")
    open(p, "w").write(str(c60["tf2d_text"][0]))
    return p


def test_c60_2dt_parses(c60, tmp_path):
    from imagevis3d_gb300 import load_tf2d_file
    w, h, tf1d, sw, ns = load_tf2d_file(_c60_2dt(c60, tmp_path))
    assert (w, h) == (256, 256) and tf1d.shape == (256, 4) and ns == 6
    first = sw[0]
    assert first.radial == 0 and first.npoints == 4 and first.nstops == 1
    assert np.allclose(list(first.points)[:8], [0.160712, 0.759697, 0.160712, 0.883628, 0.284643, 0.883628,
                                                 0.284643, 0.759697])
    assert np.allclose(list(first.stops)[:5], [0.5, 1, 0, 0, 1])
    assert sw[1].radial == 1 and sw[1].nstops == 3
    assert np.allclose(list(sw[1].grad), [0.466013, 0.509376, 0.299445, 0.394575])
    assert [sw[k].nstops for k in range(6)] == [1, 3, 3, 3, 1, 3]


def test_2dt_bad_files(tmp_path):
    from imagevis3d_gb300 import load_tf2d_file
    p = str(tmp_path / "bad.2dt")
    open(p, "w").write("4 4\n1\n0 0 0 0\n1\n0\n2\n0 0\n1 1\n")  # a 2-vertex polygon
    with pytest.raises(L.GbvrError) as e:
        load_tf2d_file(p)
    assert e.value.code == -5
    open(p, "w").write("4 4\n1\n0 0 0 0\n1\n0\n3\n0 0\n1 0\n0 1\n0 0 1 1\n2\n0.6 1 1 1 1\n0.2 0 0 0 0\n")
    with pytest.raises(L.GbvrError):
        load_tf2d_file(p)  # stops out of order


def _rect(x0, y0, x1, y1):
    return [(x0, y0), (x0, y1), (x1, y1), (x1, y0)]


def test_oracle_raster_known_answers(orc):
    # linear ramp across a rectangle; entry centres at (i + 0.5) / 8
    sw = [dict(radial=0, points=_rect(0.25, 0.25, 0.75, 0.75), grad=(0.25, 0.5, 0.75, 0.5),
               stops=[(0, 1, 0, 0, 1), (1, 0, 0, 1, 1)])]
    t = orc.raster_tf2d(sw, None, 8, 8)
    assert np.array_equal(t[2:6, 2:6, 0], np.tile([0.875, 0.625, 0.375, 0.125], (4, 1)).astype(np.float32))
    assert (t[:2, :, 3] == 0).all() and (t[6:, :, 3] == 0).all() and (t[:, :2, 3] == 0).all()
    # canvas y runs top-down, table rows bottom-up: a swatch in the top half
    # of the canvas lands in the high-gradient rows
    top = [dict(radial=0, points=_rect(0.0, 0.0, 1.0, 0.5), grad=(0, 0, 1, 0), stops=[(0, 0, 1, 0, 1)])]
    t = orc.raster_tf2d(top, None, 4, 4)
    assert (t[2:, :, 3] == 1).all() and (t[:2, :, 3] == 0).all()
    # radial: t = distance / radius, clamped
    rad = [dict(radial=1, points=_rect(0, 0, 1, 1), grad=(0.5, 0.5, 1.0, 0.5), stops=[(0, 1, 1, 1, 1), (1, 0, 0, 0, 1)])]
    t = orc.raster_tf2d(rad, None, 64, 64)
    c = np.arange(64) + 0.5
    dist = np.sqrt((c[None, :] - 32) ** 2 + (c[::-1, None] - 32) ** 2) / 32
    assert np.allclose(t[..., 0], 1 - np.minimum(dist, 1), atol=1e-6)
    # 1D TF underneath, stretched over the columns; half-transparent swatch over it
    tf1d = np.array([[1, 0, 0, 1], [0, 1, 0, 0.5]], np.float32)
    half = [dict(radial=0, points=_rect(0, 0, 1, 1), grad=(0, 0, 1, 0), stops=[(0, 0, 0, 1, 0.5)])]
    t = orc.raster_tf2d(half, tf1d, 4, 2)
    # column 0: over red (a = 1) -> a = 1, rgb = 0.5 blue + 0.5 red
    assert np.allclose(t[0, 0], [0.5, 0, 0.5, 1.0])
    # column 3: over green (a = 0.5) -> a = 0.75, rgb = (0.5 blue + 0.25 green) / 0.75
    assert np.allclose(t[0, 3], [0, 1 / 3, 2 / 3, 0.75])
    # self-intersecting bow tie: the even-odd rule leaves nothing inside twice
    bow = [dict(radial=0, points=[(0, 0), (1, 1), (1, 0), (0, 1)], grad=(0, 0, 1, 0), stops=[(0, 1, 1, 1, 1)])]
    t = orc.raster_tf2d(bow, None, 16, 16)
    assert 0.4 < t[..., 3].mean() < 0.6
