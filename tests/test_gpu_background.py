"""setBGColors with two colours (ImageVis3D/UI/RenderWindow.cpp:401-406): a
vertical gradient from the top colour at the top edge to the bottom colour at
the bottom edge, behind every 3D render mode and the 2D slice view, in the
culled batch path (background fill outside the volume's rectangle) and the
per-view path alike; against the FP64 oracle."""
import numpy as np
import pytest

from imagevis3d_gb300 import GBVR_RM_ISOSURFACE, Renderer, synth_volume, workloads
from tests.gpu_util import assert_close

pytestmark = pytest.mark.gpu

TOP = (0.9, 0.3, 0.1)
BOT = (0.05, 0.2, 0.6)


@pytest.fixture(scope="module")
def c1():
    wl = workloads.config1()
    return wl, synth_volume(wl.synth)


def test_transparent_tf_shows_the_gradient(orc, c1):
    wl, vol = c1
    w, h = 96, 64
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(wl.synth, **wl.brick)
        r.resize((w, h))
        r.set1DTrans(np.zeros((256, 4), np.float32))
        r.setValueRange(*wl.value_range)
        r.setBGColors(TOP, BOT)
        r.setView(*wl.views[0])
        r.paint()
        img = r.readFramebuffer(0, as_float=True)
        img8 = r.readFramebuffer(0)
    t = (np.arange(h) + 0.5) / h
    want = np.asarray(TOP)[None, :] + t[:, None] * (np.asarray(BOT) - np.asarray(TOP))[None, :]
    assert np.abs(img[..., :3] - want[:, None, :]).max() < 1e-6
    assert np.all(img[..., 3] == 0)
    assert np.abs(img8[..., :3].astype(np.float64) / 255 - want[:, None, :]).max() <= 0.5 / 255 + 1e-9


@pytest.mark.parametrize("mode", ["1d", "iso"])
def test_gradient_behind_the_volume_matches_oracle(orc, c1, mode):
    wl, vol = c1
    w, h = 160, 120
    views = workloads.orbit_views(3, w, h, radius=2.0 * workloads.DIAG, start=15.0)
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(wl.synth, **wl.brick)
        r.resize((w, h))
        r.set1DTrans(wl.tf)
        r.setValueRange(*wl.value_range)
        r.setBGColors(TOP, BOT)
        kw = dict(spv=wl.spv)
        if mode == "iso":
            r.setRenderMode(GBVR_RM_ISOSURFACE)
            r.setIsoValue(120.0, (0.8, 0.8, 0.9))
            kw = dict(mode=2, iso=120.0, iso_rgb=(0.8, 0.8, 0.9))
        r.paintBatch(views)   # culled tiles: the fill kernel writes the gradient outside the rectangle
        batch = [r.readFramebuffer(i, as_float=True) for i in range(len(views))]
        r.setView(*views[0])
        r.paint()
        single = r.readFramebuffer(0, as_float=True)
    assert np.array_equal(single, batch[0])
    for img, (v, p) in zip(batch, views):
        ref, _ = orc.render(vol, v, p, w, h, wl.tf, value_range=wl.value_range, bg=BOT, bg_top=TOP, **kw)
        if mode == "iso":
            hit_g, hit_r = img[..., 3] > 0.5, ref[..., 3] > 0.5
            assert (hit_g != hit_r).mean() < 0.002
            same = hit_g == hit_r
            assert_close(img[same], ref[same])
        else:
            assert_close(img, ref)


def test_gradient_behind_slices_matches_oracle(orc, c1):
    wl, vol = c1
    w, h = 128, 96
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(wl.synth, **wl.brick)
        r.resize((w, h))
        r.set1DTrans(wl.tf)
        r.setValueRange(*wl.value_range)
        r.setBGColors(TOP, BOT)
        r.paintSlice(2, 64)
        img = r.readFramebuffer(0, as_float=True)
    ref = orc.render_slice(vol, 2, 64.0, w, h, wl.tf, value_range=wl.value_range, bg=BOT, bg_top=TOP)
    assert_close(img, ref)


def test_equal_colours_are_a_flat_background(orc, c1):
    wl, vol = c1
    w, h = 64, 48
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(wl.synth, **wl.brick)
        r.resize((w, h))
        r.set1DTrans(np.zeros((256, 4), np.float32))
        r.setValueRange(*wl.value_range)
        r.setBGColors(BOT, BOT)
        r.setView(*wl.views[0])
        r.paint()
        img = r.readFramebuffer(0, as_float=True)
    assert np.all(img[..., :3] == np.float32(BOT))
