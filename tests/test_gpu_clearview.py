"""ClearView (setCV, setCVIsoValue, setCVSize, setCVContextScale,
setCVBorderScale, setCVFocusPos) in isosurface mode: the context surface
(first hit of the iso value) becomes partly transparent inside the lens over
the focus surface (first hit of the ClearView iso value behind it).

Against the FP64 oracle within the raycaster's tolerance; known answers:
outside the lens the image is the isosurface image bit for bit, and with both
scales 0 the lens shows exactly the isosurface image of the focus value."""
import numpy as np
import pytest

from imagevis3d_gb300 import GBVR_RM_ISOSURFACE, Renderer, orbit_camera, synth_params, workloads
from tests.gpu_util import assert_close

pytestmark = pytest.mark.gpu

W, H = 160, 120
ISO1, ISO2 = 60.0, 150.0
RGB1, RGB2 = (0.9, 0.75, 0.6), (0.3, 0.5, 1.0)


@pytest.fixture(scope="module")
def blobs(orc):
    sp = synth_params((72, 60, 48), np.uint8, 19, 9, (4.0, 10.0), (0.5, 1.0), 255.0, noise_kind=1, noise_amp=3.0,
                      vmax=255.0)
    return sp, orc.synth_blobs(sp)


def _renderer(sp, iso=ISO1, rgb=RGB1, lighting=True, float_fb=True):
    r = Renderer(float_fb=float_fb)
    r.loadSynthetic(sp, brick_size=32, overlap=2)
    r.resize((W, H))
    r.setRenderMode(GBVR_RM_ISOSURFACE)
    r.set1DTrans(workloads.tf1d_seeded(256, 19, 30.0, 255.0))
    r.setValueRange(0.0, 255.0)
    r.setIsoValue(iso, rgb)
    if not lighting:
        r.setLightingEnabled(False)
    return r


def _cv(r, fx=W / 2, fy=H / 2, size=0.8, context=1.0, border=1.0):
    r.setCVIsoValue(ISO2)
    r.setCVColor(RGB2)
    r.setCVSize(size)
    r.setCVContextScale(context)
    r.setCVBorderScale(border)
    r.setCVFocusPos(fx, fy)
    r.setCV(True)


def _paint(r, cam):
    r.setView(*cam)
    r.paint()
    return r.readFramebuffer(0, as_float=True)


def _lens_mask(fx, fy, radius):
    yy, xx = np.mgrid[0:H, 0:W]
    return np.hypot(xx + 0.5 - fx, yy + 0.5 - fy) / radius < 1.0


CAMS = [orbit_camera(30.0, 20.0, 2.2 * workloads.DIAG, 45.0, W, H),
        orbit_camera(210.0, -35.0, 1.6 * workloads.DIAG, 45.0, W, H)]


@pytest.mark.parametrize("cam", [0, 1])
@pytest.mark.parametrize("scales", [(1.0, 1.0), (0.6, 2.0), (1.5, 0.3)])
def test_clearview_vs_oracle(orc, blobs, cam, scales):
    sp, vol = blobs
    with _renderer(sp) as r:
        _cv(r, context=scales[0], border=scales[1])
        img = _paint(r, CAMS[cam])
    radius = float(np.float32(0.8 * 0.5 * min(W, H)))
    ref, _ = orc.render(vol, *CAMS[cam], W, H, workloads.tf1d_seeded(256, 19, 30.0, 255.0), value_range=(0.0, 255.0),
                        mode=2, iso=ISO1, iso_rgb=RGB1,
                        cv=dict(iso=ISO2, rgb=RGB2, context=scales[0], border=scales[1], focus=(W / 2, H / 2),
                                radius=radius))
    assert_close(img, ref)


def test_outside_the_lens_is_the_isosurface_image(blobs):
    sp, _ = blobs
    fx, fy, size = 50.0, 70.0, 0.5
    with _renderer(sp) as a, _renderer(sp) as b:
        _cv(b, fx, fy, size)
        ia, ib = _paint(a, CAMS[0]), _paint(b, CAMS[0])
    lens = _lens_mask(fx, fy, size * 0.5 * min(W, H))
    assert np.array_equal(ia[~lens], ib[~lens])
    assert not np.array_equal(ia[lens], ib[lens])  # the lens shows the focus surface


def test_transparent_context_shows_the_focus_isosurface(blobs):
    """Both scales 0: the context surface is fully transparent in the lens,
    which then holds the isosurface image of the focus value (the focus
    value is the higher one, so its first crossing lies behind)."""
    sp, _ = blobs
    for cam in CAMS:
        with _renderer(sp) as a, _renderer(sp, iso=ISO2, rgb=RGB2) as b:
            _cv(a, context=0.0, border=0.0)
            ia, ib = _paint(a, cam), _paint(b, cam)
        lens = _lens_mask(W / 2, H / 2, 0.8 * 0.5 * min(W, H))
        assert np.array_equal(ia[lens], ib[lens])
        assert (ib[lens][:, 3] == 1.0).sum() > 200


def test_lens_off_screen_and_off(blobs):
    sp, _ = blobs
    with _renderer(sp) as a, _renderer(sp) as b:
        _cv(b, fx=-500.0, fy=-500.0, size=0.5)
        base = _paint(a, CAMS[1])
        assert np.array_equal(base, _paint(b, CAMS[1]))
        _cv(b)
        assert not np.array_equal(base, _paint(b, CAMS[1]))
        b.setCV(False)
        assert np.array_equal(base, _paint(b, CAMS[1]))


def test_batch_equals_per_view_with_lines(orc, blobs):
    sp, vol = blobs
    views = workloads.orbit_views(6, W, H, elevation=15.0)
    with _renderer(sp, float_fb=False) as r:
        _cv(r)
        r.setGlobalBBox(True)
        r.setLocalBBox(True)
        r.paintBatch(views)
        batch = r.readFramebuffers(0, 6)
        r.paintViews(views)
        assert np.array_equal(batch, r.readFramebuffers(0, 6))
    # lines inside the lens against the oracle
    with _renderer(sp) as r:
        _cv(r)
        r.setGlobalBBox(True)
        r.setLocalBBox(True)
        img = _paint(r, views[2])
    radius = float(np.float32(0.8 * 0.5 * min(W, H)))
    ref, _ = orc.render(vol, *views[2], W, H, workloads.tf1d_seeded(256, 19, 30.0, 255.0), value_range=(0.0, 255.0),
                        mode=2, iso=ISO1, iso_rgb=RGB1, bbox=dict(global_=True, local=True, interior=28),
                        cv=dict(iso=ISO2, rgb=RGB2, focus=(W / 2, H / 2), radius=radius))
    assert_close(img, ref)
