"""2D transfer functions from .2dt swatches: the GPU rasteriser equals the
oracle's restatement bit for bit, and a renderer given the file renders as it
does with the rasterised table."""
import numpy as np
import pytest

from imagevis3d_gb300 import (GBVR_RM_2DTRANS, Renderer, load_tf2d_file, orbit_camera, synth_params, tf2d_rasterize,
                              workloads)
from imagevis3d_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _to_dicts(sw, ns):
    out = []
    for k in range(ns):
        s = sw[k]
        out.append(dict(radial=s.radial, points=[(s.points[2 * j], s.points[2 * j + 1]) for j in range(s.npoints)],
                        grad=tuple(s.grad), stops=[tuple(s.stops[5 * j:5 * j + 5]) for j in range(s.nstops)]))
    return out


@pytest.fixture()
def c60_2dt(c60, tmp_path):
    p = str(tmp_path / "c60.2dt")
    open(p, "w").write(str(c60["tf2d_text"][0]))
    return p


@pytest.mark.parametrize("size", [(256, 256), (300, 64), (17, 101)])
def test_c60_swatches_match_oracle(orc, c60_2dt, size):
    w, h, tf1d, sw, ns = load_tf2d_file(c60_2dt)
    got = tf2d_rasterize(sw, ns, tf1d, *size)
    want = orc.raster_tf2d(_to_dicts(sw, ns), tf1d, *size)
    assert np.array_equal(got, want)
    assert got[..., 3].max() > 0.5


def _random_swatches(rng, n):
    out = []
    for _ in range(n):
        k = int(rng.integers(3, 13))
        cx, cy = rng.uniform(-0.1, 1.1, 2)
        ang = np.sort(rng.uniform(0, 2 * np.pi, k)) if rng.random() < 0.7 else rng.uniform(0, 2 * np.pi, k)
        rad = rng.uniform(0.05, 0.5, k)
        pts = [(float(cx + r * np.cos(a)), float(cy + r * np.sin(a))) for a, r in zip(ang, rad)]
        ns = int(rng.integers(1, 17))
        pos = np.sort(rng.uniform(0, 1, ns))
        if rng.random() < 0.3 and ns > 2:
            pos[1] = pos[0]  # a repeated stop position
        stops = [(float(p),) + tuple(float(x) for x in rng.uniform(0, 1, 4)) for p in pos]
        g = tuple(float(x) for x in rng.uniform(-0.2, 1.2, 4))
        out.append(dict(radial=int(rng.random() < 0.4), points=pts, grad=g, stops=stops))
    return out


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_swatches_match_oracle(orc, seed):
    rng = np.random.default_rng(seed)
    sws = _random_swatches(rng, 24)
    tf1d = rng.uniform(0, 1, (int(rng.integers(2, 300)), 4)).astype(np.float32)
    arr = orc.make_swatches(sws)
    swc = (L.Tf2dSwatch * len(sws)).from_buffer_copy(bytes(arr))
    for size in [(256, 256), (129, 77)]:
        got = tf2d_rasterize(swc, len(sws), tf1d, *size)
        want = orc.raster_tf2d(sws, tf1d, *size)
        assert np.array_equal(got, want)
    # no 1D TF: transparent black underneath
    got = tf2d_rasterize(swc, len(sws), None, 64, 64)
    assert np.array_equal(got, orc.raster_tf2d(sws, None, 64, 64))


def test_rasterize_rejects_bad_swatches(orc):
    sw = orc.make_swatches([dict(radial=0, points=[(0, 0), (1, 0), (0, 1)], grad=(0, 0, 1, 0),
                                 stops=[(0.5, 1, 1, 1, 1), (0.2, 0, 0, 0, 1)])])
    swc = (L.Tf2dSwatch * 1).from_buffer_copy(bytes(sw))
    with pytest.raises(L.GbvrError):
        tf2d_rasterize(swc, 1, None, 8, 8)


def test_renderer_takes_the_2dt_file(c60_2dt):
    sp = synth_params((96, 80, 72), np.uint8, 3, 8, (4.0, 10.0), (0.3, 1.0), 255.0, noise_kind=1, noise_amp=4.0,
                      vmax=255.0)
    view, proj = orbit_camera(30.0, 20.0, 2.5 * workloads.DIAG, 45.0, 96, 80)
    w, h, tf1d, sw, ns = load_tf2d_file(c60_2dt)
    table = tf2d_rasterize(sw, ns, tf1d, w, h)
    imgs = []
    for use_file in (True, False):
        with Renderer(float_fb=True) as r:
            r.loadSynthetic(sp, brick_size=64, overlap=2)
            r.resize((96, 80))
            r.setRenderMode(GBVR_RM_2DTRANS)
            if use_file:
                r.set2DTransFile(c60_2dt, 0.0)
            else:
                r.set2DTrans(table, 0.0)
            r.setView(view, proj)
            r.paint()
            imgs.append(r.readFramebuffer(0, as_float=True))
    assert np.array_equal(imgs[0], imgs[1])
