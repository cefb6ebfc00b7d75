"""Edge cases of the raycaster against the FP64 oracle: non-unit voxel aspect,
ragged and tiny framebuffers, a one-voxel-thick slab, sampling rates below
and above one sample per voxel, early-termination thresholds, a coloured
background, orthographic projection, batches of 100 and 4096 views against
the per-view launches, and an 8192 x 8192 framebuffer."""
import numpy as np
import pytest

from imagevis3d_gb300 import GBVR_RM_1DTRANS, GBVR_RM_ISOSURFACE, Renderer, orbit_camera, synth_params, workloads
from tests.gpu_util import assert_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def blobs(orc):
    sp = synth_params((72, 60, 48), np.uint8, 17, 7, (3.0, 9.0), (0.3, 1.0), 255.0, noise_kind=1, noise_amp=4.0,
                      vmax=255.0)
    return sp, orc.synth_blobs(sp)


TF = workloads.tf1d_seeded(256, 17, 30.0, 255.0)


def _render(sp, view, proj, w, h, aspect=None, spv=1.0, ert=0.99, bg=(0, 0, 0), mode=GBVR_RM_1DTRANS, iso=0.0):
    with Renderer(float_fb=True) as r:
        kw = dict(brick_size=32, overlap=2)
        if aspect is not None:
            kw["aspect"] = aspect
        r.loadSynthetic(sp, **kw)
        r.resize((w, h))
        r.setRenderMode(mode)
        r.set1DTrans(TF)
        r.setValueRange(0.0, 255.0)
        r.setSampleRateModifier(spv)
        r.setEarlyTermination(ert)
        r.setBGColors(bg, bg)
        r.setIsoValue(iso)
        r.setView(view, proj)
        r.paint()
        return r.readFramebuffer(0, as_float=True)


def _oracle(orc, vol, view, proj, w, h, **kw):
    ref, _ = orc.render(vol, view, proj, w, h, TF, value_range=(0.0, 255.0), **kw)
    return ref


def test_non_unit_aspect(orc, blobs):
    sp, vol = blobs
    aspect = (1.0, 1.5, 2.5)
    view, proj = orbit_camera(40.0, 25.0, 2.5 * workloads.DIAG, 45.0, 160, 120)
    img = _render(sp, view, proj, 160, 120, aspect=aspect)
    ext = np.array([72 * 1.0, 60 * 1.5, 48 * 2.5])
    ext = ext / ext.max()
    assert_close(img, _oracle(orc, vol, view, proj, 160, 120, extent=tuple(ext)))


@pytest.mark.parametrize("size", [(1, 1), (3, 5), (7, 33), (37, 2)])
def test_tiny_and_ragged_framebuffers(orc, blobs, size):
    sp, vol = blobs
    w, h = size
    view, proj = orbit_camera(20.0, 10.0, 1.2 * workloads.DIAG, 30.0, w, h)  # close: the volume fills the frame
    img = _render(sp, view, proj, w, h)
    assert img.shape == (h, w, 4)
    assert_close(img, _oracle(orc, vol, view, proj, w, h))


def test_one_voxel_thick_slab(orc):
    sp = synth_params((64, 48, 1), np.uint8, 3, 5, (3.0, 9.0), (0.5, 1.0), 255.0, noise_kind=1, noise_amp=4.0,
                      vmax=255.0)
    vol = orc.synth_blobs(sp)
    view, proj = orbit_camera(10.0, 60.0, 2.0, 45.0, 128, 96)
    img = _render(sp, view, proj, 128, 96)
    ref = _oracle(orc, vol, view, proj, 128, 96)
    assert_close(img, ref)


@pytest.mark.parametrize("spv", [0.5, 3.0])
def test_sampling_rates(orc, blobs, spv):
    sp, vol = blobs
    view, proj = orbit_camera(110.0, -15.0, 2.5 * workloads.DIAG, 45.0, 128, 96)
    img = _render(sp, view, proj, 128, 96, spv=spv)
    assert_close(img, _oracle(orc, vol, view, proj, 128, 96, spv=spv))


@pytest.mark.parametrize("ert", [0.5, 1.0])
def test_early_termination_and_background(orc, blobs, ert):
    sp, vol = blobs
    bg = (0.25, 0.5, 0.75)
    view, proj = orbit_camera(200.0, 30.0, 2.5 * workloads.DIAG, 45.0, 128, 96)
    img = _render(sp, view, proj, 128, 96, ert=ert, bg=bg)
    assert_close(img, _oracle(orc, vol, view, proj, 128, 96, ert=ert, bg=bg))


def _ortho(width, height, half_h, znear, zfar):
    a = width / height
    P = np.zeros((4, 4), np.float32)
    P[0, 0] = 1.0 / (half_h * a)
    P[1, 1] = 1.0 / half_h
    P[2, 2] = -2.0 / (zfar - znear)
    P[2, 3] = -(zfar + znear) / (zfar - znear)
    P[3, 3] = 1.0
    return P


@pytest.mark.parametrize("mode", [GBVR_RM_1DTRANS, GBVR_RM_ISOSURFACE])
def test_orthographic_projection(orc, blobs, mode):
    sp, vol = blobs
    view, _ = orbit_camera(60.0, 35.0, 3.0, 45.0, 160, 120)
    proj = _ortho(160, 120, 0.7, 0.5, 6.0)
    img = _render(sp, view, proj, 160, 120, mode=mode, iso=120.0)
    ref = _oracle(orc, vol, view, proj, 160, 120, mode=mode, iso=120.0)
    assert_close(img, ref)
    assert ref[..., 3].max() > 0.3


def test_large_batch_equals_per_view_launches(blobs):
    sp, _ = blobs
    views = workloads.orbit_views(100, 96, 72, elevation=15.0)
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(sp, brick_size=32, overlap=2)
        r.resize((96, 72))
        r.set1DTrans(TF)
        r.setValueRange(0.0, 255.0)
        r.paintBatch(views)
        batch = r.readFramebuffers(0, 100)
        r.paintViews(views)
        plain = r.readFramebuffers(0, 100)
        assert np.array_equal(batch, plain)
        r.setView(*views[37])
        r.paint()
        assert np.array_equal(r.readFramebuffer(0), batch[37])


def test_batches_of_new_views_replay_the_cached_graph(blobs):
    """Same-sized batches replay one cached launch; each new set of views
    culls to a different tile count, which the replay must follow."""
    sp, _ = blobs
    steps = [workloads.orbit_views(4, 96, 72, elevation=e, start=s) for e, s in ((5, 0), (25, 30), (-35, 60), (15, 90))]
    with Renderer() as r:
        r.loadSynthetic(sp, brick_size=32, overlap=2)
        r.resize((96, 72))
        r.set1DTrans(TF)
        r.setValueRange(0.0, 255.0)
        for views in steps:
            r.paintBatch(views)
            batch = r.readFramebuffers(0, 4).copy()
            r.paintViews(views)
            assert np.array_equal(batch, r.readFramebuffers(0, 4))


def test_many_small_views_in_one_batch(blobs):
    """4096 views in one persistent launch equal the per-view launches."""
    sp, _ = blobs
    views = workloads.orbit_views(4096, 32, 24, elevation=25.0)
    with Renderer() as r:
        r.loadSynthetic(sp, brick_size=32, overlap=2)
        r.resize((32, 24))
        r.set1DTrans(TF)
        r.setValueRange(0.0, 255.0)
        r.paintBatch(views)
        batch = r.readFramebuffers(0, 4096)
        r.paintViews(views)
        assert np.array_equal(batch, r.readFramebuffers(0, 4096))
        assert (batch[..., 3] > 0).any(axis=(1, 2)).all()


def test_large_framebuffer(orc, blobs):
    """One 8192 x 8192 view: the persistent and the per-view kernel agree bit
    for bit, and seeded pixels match the oracle."""
    sp, vol = blobs
    w = h = 8192
    view, proj = orbit_camera(70.0, 20.0, 1.8 * workloads.DIAG, 45.0, w, h)
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(sp, brick_size=32, overlap=2)
        r.resize((w, h))
        r.set1DTrans(TF)
        r.setValueRange(0.0, 255.0)
        r.paintBatch([(view, proj)])
        batch = r.readFramebuffer(0, as_float=True)
        r.setView(view, proj)
        r.paint()
        img = r.readFramebuffer(0, as_float=True)
    assert np.array_equal(batch, img)
    pix = np.random.default_rng(3).choice(w * h, 20000, replace=False)
    ref, _ = orc.render(vol, view, proj, w, h, TF, value_range=(0.0, 255.0), pixels=pix)
    assert_close(img.reshape(-1, 4)[pix], ref)
    assert (ref[:, 3] > 0).sum() > 1000
