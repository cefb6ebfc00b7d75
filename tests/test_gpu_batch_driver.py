"""The headless C++ driver gbvr_batch replays LuaScripts/BatchRenderer.lua
(new renderer, loadDataset, resize, paint, captureSingleFrame, cleanup) and
writes the same pixels the library renders."""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

from imagevis3d_gb300 import Renderer, orbit_camera
from tests.test_tf_files import _write_1dt
from tests.test_uvf_host import write_c60

pytestmark = pytest.mark.gpu
DRIVER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "imagevis3d_gb300", "gbvr_batch")


def read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w = 8, b"", 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            ch = 4 if ctype == 6 else 3
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + w * ch)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, ch)


def test_driver_single_frame_and_orbit(c60, tmp_path):
    uvf = str(tmp_path / "c60.uvf")
    write_c60(c60, uvf)
    tf = str(tmp_path / "c60.1dt")
    _write_1dt(tf, c60["tf1d"])
    out = str(tmp_path / "render.png")
    p = subprocess.run([DRIVER, "-f", uvf, "-o", out, "-tf", tf, "-size", "160", "120"], capture_output=True,
                       text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    img = read_png(out)
    with Renderer() as r:
        r.loadDataset(uvf)
        r.set1DTrans(c60["tf1d"])
        r.resize((160, 120))
        r.setView(*orbit_camera(0.0, 20.0, 2.5 * 3 ** 0.5, 45.0, 160, 120))
        r.paint()
        want = r.readFramebuffer(0)
    assert np.array_equal(img, want)
    assert img[..., 3].max() > 0
    p = subprocess.run([DRIVER, "-f", uvf, "-o", str(tmp_path / "orbit.png"), "-tf", tf, "-size", "64", "48",
                        "-views", "4"], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    frames = [read_png(str(tmp_path / ("orbit_%04d.png" % i))) for i in range(4)]
    assert all(f.shape == (48, 64, 4) for f in frames)
    assert not np.array_equal(frames[0], frames[1])


def test_driver_reports_bad_input(tmp_path):
    bad = str(tmp_path / "bad.uvf")
    open(bad, "wb").write(b"nope")
    p = subprocess.run([DRIVER, "-f", bad, "-o", str(tmp_path / "x.png")], capture_output=True, text=True,
                       timeout=120)
    assert p.returncode == 1 and "loadDataset" in p.stderr
