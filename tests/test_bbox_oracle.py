"""Bounding-box line rule of the oracle (CPU): known answers for an
orthographic view down the z axis, where every projected box edge lands at a
known pixel position."""
import numpy as np

from oracle import orc

W, H = 40, 30


def _ortho_down_z():
    view = np.eye(4, dtype=np.float32)
    view[2, 3] = -3.0  # eye at z = +3 looking down -z
    P = np.zeros((4, 4), np.float32)
    P[0, 0] = 1 / 0.6
    P[1, 1] = 1 / 0.45
    P[2, 2] = -2 / (10 - 0.5)
    P[2, 3] = -(10 + 0.5) / (10 - 0.5)
    P[3, 3] = 1
    return view, P


def _decode(keys):
    z = (keys & ~np.uint32(1)).view(np.float32).astype(np.float64) - 2.0
    return z, keys & 1


def test_global_box_edges_known_columns():
    view, P = _ortho_down_z()
    k = orc.line_keys((64, 64, 64), (1.0, 1.0, 1.0), view, P, W, H, dict(global_=True))
    cov = k != 0xFFFFFFFF
    # x = -0.5 and +0.5 project to 3.33 and 36.67 pixels: columns 3 and 36,
    # every row (the box's y edges lie outside the 0.45-high view)
    want = np.zeros((H, W), bool)
    want[:, 3] = want[:, 36] = True
    assert np.array_equal(cov, want)
    z, color = _decode(k[cov])
    assert (color == 0).all()
    # the nearer (front, z = +0.5) edges win: eye distance 2.5
    z_front = (-2 / 9.5) * -2.5 - 10.5 / 9.5
    assert np.allclose(z, z_front, atol=1e-6)


def test_brick_grid_lines_and_ties():
    view, P = _ortho_down_z()
    # 64^3 with interior 32: one interior bound per axis at x = 0 (pixel 20.0)
    k = orc.line_keys((64, 64, 64), (1.0, 1.0, 1.0), view, P, W, H,
                      dict(global_=True, local=True, interior=32))
    cov = k != 0xFFFFFFFF
    # centres 19.5 and 20.5 are exactly half a pixel from x = 20: both covered
    for c in (3, 19, 20, 36):
        assert cov[:, c].all(), c
    # the horizontal grid line y = 0 projects to row 15.0 between columns
    # 3.33 and 36.67: rows 14 and 15, columns 3 .. 36
    for r in (14, 15):
        assert cov[r, 3:37].all() and not cov[r, :3].any() and not cov[r, 37:].any()
    other = np.ones(W, bool)
    other[[3, 19, 20, 36]] = False
    assert not cov[:14][:, other].any()
    _, color = _decode(k)
    assert (color[:, 3] == 0).all() and (color[:, 19] == 1).all()


def test_local_box_alone_keeps_outer_edges():
    view, P = _ortho_down_z()
    k = orc.line_keys((64, 64, 64), (1.0, 1.0, 1.0), view, P, W, H, dict(local=True, interior=32))
    _, color = _decode(k)
    cov = k != 0xFFFFFFFF
    assert cov[:, 3].all() and cov[:, 36].all()
    assert (color[cov] == 1).all()


def test_no_lines_behind_the_eye():
    # the camera inside the box: segments are clipped to the near plane, and a
    # box entirely behind the eye draws nothing
    view = np.eye(4, dtype=np.float32)
    view[2, 3] = 5.0  # eye at z = -5 looking down -z: the box is behind it
    P = np.zeros((4, 4), np.float32)
    f = 1 / np.tan(np.radians(22.5))
    P[0, 0], P[1, 1] = f * H / W, f
    P[2, 2], P[2, 3], P[3, 2] = -(10.1) / 9.9, -2 * 10 * 0.1 / 9.9, -1
    k = orc.line_keys((64, 64, 64), (1.0, 1.0, 1.0), view, P, W, H, dict(global_=True))
    assert (k == 0xFFFFFFFF).all()
