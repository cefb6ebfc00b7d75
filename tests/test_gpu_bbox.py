"""Bounding-box lines (setGlobalBBox / setLocalBBox) against the FP64 oracle:
with a transparent volume the image is exactly the lines over the background
(coverage and colour bit for bit); with a visible volume the images agree
within the raycaster's tolerance in 1D, isosurface and MIP modes, with the
eye inside the volume and with an orthographic camera; batched = per-view."""
import numpy as np
import pytest

from imagevis3d_gb300 import (GBVR_RM_1DTRANS, GBVR_RM_ISOSURFACE, GBVR_RM_MIP, Renderer, look_at_camera,
                              orbit_camera, synth_params, workloads)
from tests.gpu_util import assert_close

pytestmark = pytest.mark.gpu

BRICK, GHOST = 32, 2
TF = workloads.tf1d_seeded(256, 17, 30.0, 255.0)
RGB = ((1.0, 0.9, 0.2), (0.3, 0.5, 1.0))


@pytest.fixture(scope="module")
def blobs(orc):
    sp = synth_params((72, 60, 48), np.uint8, 17, 7, (3.0, 9.0), (0.3, 1.0), 255.0, noise_kind=1, noise_amp=4.0,
                      vmax=255.0)
    return sp, orc.synth_blobs(sp)


def _renderer(sp, w, h, g, l, mode=GBVR_RM_1DTRANS, tf=TF, iso=120.0):
    r = Renderer(float_fb=True)
    r.loadSynthetic(sp, brick_size=BRICK, overlap=GHOST)
    r.resize((w, h))
    r.setRenderMode(mode)
    r.set1DTrans(tf)
    r.setValueRange(0.0, 255.0)
    r.setIsoValue(iso)
    r.setGlobalBBox(g, RGB[0])
    r.setLocalBBox(l, RGB[1])
    return r


def _oracle(orc, vol, view, proj, w, h, g, l, tf=TF, **kw):
    ref, _ = orc.render(vol, view, proj, w, h, tf, value_range=(0.0, 255.0),
                        bbox=dict(global_=g, local=l, interior=BRICK - 2 * GHOST, rgb=RGB), **kw)
    return ref


def _inside_camera(w, h):
    # looking along +x from inside the volume, slightly off axis
    return look_at_camera((-0.3, 0.05, 0.02), (0.5, -0.02, 0.1), (0, 1, 0), 50.0, w, h)


CAMS = {
    "orbit": lambda w, h: orbit_camera(35.0, 25.0, 2.2 * workloads.DIAG, 45.0, w, h),
    "close": lambda w, h: orbit_camera(200.0, -30.0, 1.1 * workloads.DIAG, 45.0, w, h),
    "inside": _inside_camera,
}


@pytest.mark.parametrize("cam", sorted(CAMS))
@pytest.mark.parametrize("g,l", [(True, False), (False, True), (True, True)])
def test_lines_over_transparent_volume_exact(orc, blobs, cam, g, l):
    sp, vol = blobs
    w, h = 160, 120
    view, proj = CAMS[cam](w, h)
    empty = np.zeros_like(TF)
    with _renderer(sp, w, h, g, l, tf=empty) as r:
        r.setView(view, proj)
        r.paint()
        img = r.readFramebuffer(0, as_float=True)
    ref = _oracle(orc, vol, view, proj, w, h, g, l, tf=empty)
    assert np.array_equal(img[..., 3] == 1.0, ref[..., 3] == 1.0)
    assert np.array_equal(img.astype(np.float64), ref.astype(np.float32).astype(np.float64))
    assert (img[..., 3] == 1.0).sum() > 100


@pytest.mark.parametrize("mode", [GBVR_RM_1DTRANS, GBVR_RM_ISOSURFACE, GBVR_RM_MIP])
@pytest.mark.parametrize("cam", ["orbit", "inside"])
def test_lines_with_volume_vs_oracle(orc, blobs, mode, cam):
    sp, vol = blobs
    w, h = 160, 120
    view, proj = CAMS[cam](w, h)
    with _renderer(sp, w, h, True, True, mode=mode) as r:
        r.setView(view, proj)
        r.paint()
        img = r.readFramebuffer(0, as_float=True)
    ref = _oracle(orc, vol, view, proj, w, h, True, True, mode=mode, iso=120.0)
    assert_close(img, ref)
    # lines behind the volume show through where it is not opaque
    assert (ref[..., 3] == 1.0).sum() > 100


def test_orthographic_lines(orc, blobs):
    sp, vol = blobs
    w, h = 128, 96
    view, _ = orbit_camera(60.0, 35.0, 3.0, 45.0, w, h)
    a = w / h
    P = np.zeros((4, 4), np.float32)
    P[0, 0], P[1, 1] = 1.0 / (0.7 * a), 1.0 / 0.7
    P[2, 2], P[2, 3], P[3, 3] = -2.0 / 5.5, -6.5 / 5.5, 1.0
    with _renderer(sp, w, h, True, True) as r:
        r.setView(view, P)
        r.paint()
        img = r.readFramebuffer(0, as_float=True)
    assert_close(img, _oracle(orc, vol, view, P, w, h, True, True))


def test_batch_equals_per_view_and_lines_off(blobs):
    sp, _ = blobs
    views = workloads.orbit_views(12, 96, 72, elevation=20.0)
    with _renderer(sp, 96, 72, True, True) as r:
        r.paintBatch(views)
        batch = r.readFramebuffers(0, 12)
        r.paintViews(views)
        assert np.array_equal(batch, r.readFramebuffers(0, 12))
        r.setView(*views[5])
        r.paint()
        assert np.array_equal(r.readFramebuffer(0), batch[5])
        # switched off: the plain images again
        r.setGlobalBBox(False)
        r.setLocalBBox(False)
        r.paintBatch(views)
        off = r.readFramebuffers(0, 12)
    with _renderer(sp, 96, 72, False, False) as r:
        r.paintBatch(views)
        assert np.array_equal(off, r.readFramebuffers(0, 12))
    assert not np.array_equal(off, batch)


def test_lines_at_a_coarser_level(orc, blobs):
    """The brick grid drawn is the rendered level's (LOD 1 of 72x60x48 is
    36x30x24: 2 x 2 x 1 bricks of interior 28)."""
    sp, vol = blobs
    w, h = 128, 96
    view, proj = CAMS["orbit"](w, h)
    with _renderer(sp, w, h, False, True) as r:
        r.setLODLimits(1, 8)
        r.setView(view, proj)
        r.paint()
        img = r.readFramebuffer(0, as_float=True)
    lv1 = orc.downsample(vol)
    ext = (72 / 72, 60 / 72, 48 / 72)  # the finest level's box
    ref = _oracle(orc, lv1, view, proj, w, h, False, True, extent=ext)
    assert_close(img, ref)
