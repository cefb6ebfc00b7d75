"""Maximum-intensity projection and the clip plane against the FP64 oracle.

MIP skips bricks and macro-cells whose largest voxel cannot raise the running
maximum, and stops at the level's maximum: every skipping mode must give the
same image bit for bit.  The clip plane cuts each ray's sample range without
moving the samples."""
import numpy as np
import pytest

from imagevis3d_gb300 import (GBVR_RM_1DTRANS, GBVR_RM_2DTRANS, GBVR_RM_ISOSURFACE, GBVR_RM_MIP, Renderer,
                              orbit_camera, synth_params, workloads)
from tests.gpu_util import assert_close

pytestmark = pytest.mark.gpu

DIMS = (150, 130, 110)
W, H = 200, 150


@pytest.fixture(scope="module")
def vol_u16(orc):
    sp = synth_params(DIMS, np.uint16, 11, 10, (4.0, 12.0), (0.3, 1.0), 2600.0, noise_kind=2, noise_amp=20.0,
                      vmax=4095.0, bg_freq=1.0, bg_level=0.15, bg_amp=0.1)
    return sp, orc.synth_blobs(sp)


def _renderer(sp, mode, tf, rng=(0.0, 4095.0), **bp):
    r = Renderer(float_fb=True)
    r.loadSynthetic(sp, brick_size=64, overlap=2, **bp)
    r.resize((W, H))
    r.setRenderMode(mode)
    r.set1DTrans(tf)
    r.setValueRange(*rng)
    r.setSampleRateModifier(1.0)
    return r


def _paint(r, view, proj):
    r.setView(view, proj)
    r.paint()
    return r.readFramebuffer(0, as_float=True)


VIEWS = [(35.0, 20.0), (160.0, -40.0), (280.0, 65.0)]


@pytest.mark.parametrize("az,el", VIEWS)
def test_mip_matches_oracle(orc, vol_u16, az, el):
    sp, vol = vol_u16
    tf = workloads.tf1d_seeded(4096, 7, 500.0, 4095.0)
    view, proj = orbit_camera(az, el, 2.5 * workloads.DIAG, 45.0, W, H)
    with _renderer(sp, GBVR_RM_MIP, tf) as r:
        img = _paint(r, view, proj)
    ref, _ = orc.render(vol, view, proj, W, H, tf, spv=1.0, value_range=(0.0, 4095.0), mode=3)
    assert_close(img, ref)
    assert ref[..., 3].max() > 0.5


def test_mip_skipping_is_exact_and_batch_equals_plain(vol_u16):
    sp, _ = vol_u16
    tf = workloads.tf1d_seeded(4096, 7, 500.0, 4095.0)
    views = [orbit_camera(az, el, 2.5 * workloads.DIAG, 45.0, W, H) for az, el in VIEWS]
    with _renderer(sp, GBVR_RM_MIP, tf) as r:
        imgs = {}
        for mode in (0, 1, 2):
            r.setEmptySkipping(mode)
            imgs[mode] = [_paint(r, v, p) for v, p in views]
            st = r.stats()
            imgs[(mode, "samples")] = st["samples"]
        for i in range(len(views)):
            assert np.array_equal(imgs[0][i], imgs[1][i]) and np.array_equal(imgs[0][i], imgs[2][i])
        # the running-maximum skips take fewer samples
        assert imgs[(2, "samples")] < imgs[(0, "samples")]
        r.paintBatch(views)
        for i in range(len(views)):
            assert np.array_equal(r.readFramebuffer(i, as_float=True), imgs[2][i])


def test_mip_lod1_and_u8(orc):
    sp = synth_params((120, 90, 100), np.uint8, 4, 8, (3.0, 9.0), (0.3, 1.0), 255.0, noise_kind=1, noise_amp=4.0,
                      vmax=255.0)
    vol = orc.synth_blobs(sp)
    tf = workloads.tf1d_seeded(256, 4, 30.0, 255.0)
    view, proj = orbit_camera(60.0, 25.0, 2.5 * workloads.DIAG, 45.0, W, H)
    with _renderer(sp, GBVR_RM_MIP, tf, rng=(0.0, 255.0)) as r:
        img0 = _paint(r, view, proj)
        r.setLODLimits(1, 1)
        img1 = _paint(r, view, proj)
    ref0, _ = orc.render(vol, view, proj, W, H, tf, spv=1.0, value_range=(0.0, 255.0), mode=3)
    assert_close(img0, ref0)
    ref1, _ = orc.render(orc.downsample(vol), view, proj, W, H, tf, spv=1.0, value_range=(0.0, 255.0), mode=3,
                         extent=(120 / 120, 90 / 120, 100 / 120))
    assert_close(img1, ref1)


def test_mip_supercell_skips_on_a_clean_background(orc):
    """Blobs on an empty background: once a ray has crossed a blob, whole
    super-cells of 4^3 macro-cells fall below its maximum and are left at
    once.  Every skipping mode gives the same image bit for bit, and the
    oracle agrees; the skips take far fewer samples."""
    sp = synth_params((160, 144, 128), np.uint16, 21, 12, (4.0, 10.0), (0.4, 1.0), 3000.0, vmax=4095.0)
    vol = orc.synth_blobs(sp)
    tf = workloads.tf1d_seeded(4096, 21, 200.0, 4095.0)
    view, proj = orbit_camera(50.0, 30.0, 2.5 * workloads.DIAG, 45.0, W, H)
    with _renderer(sp, GBVR_RM_MIP, tf) as r:
        imgs, samples = {}, {}
        for mode in (0, 2):
            r.setEmptySkipping(mode)
            imgs[mode] = _paint(r, view, proj)
            samples[mode] = r.stats()["samples"]
    assert np.array_equal(imgs[0], imgs[2])
    assert samples[2] < 0.5 * samples[0]
    ref, _ = orc.render(vol, view, proj, W, H, tf, spv=1.0, value_range=(0.0, 4095.0), mode=3)
    assert_close(imgs[2], ref)
    assert ref[..., 3].max() > 0.3


PLANES = [(1.0, 0.0, 0.0, 0.1), (-0.3, 0.8, 0.5, 0.05), (0.0, 0.0, -1.0, -0.2)]


@pytest.mark.parametrize("plane", PLANES)
@pytest.mark.parametrize("mode", [GBVR_RM_1DTRANS, GBVR_RM_ISOSURFACE, GBVR_RM_MIP])
def test_clip_plane_matches_oracle(orc, vol_u16, plane, mode):
    sp, vol = vol_u16
    tf = workloads.tf1d_seeded(4096, 11, 900.0, 4095.0)
    view, proj = orbit_camera(35.0, 20.0, 2.5 * workloads.DIAG, 45.0, W, H)
    with _renderer(sp, mode, tf) as r:
        r.setIsoValue(1300.0)
        full = _paint(r, view, proj)
        r.setClipPlane(plane)
        img = _paint(r, view, proj)
        # the plane only ever removes samples: skipping modes stay exact
        r.setEmptySkipping(0)
        assert np.array_equal(_paint(r, view, proj), img)
        r.setEmptySkipping(2)
        r.setClipPlane(None)
        assert np.array_equal(_paint(r, view, proj), full)
    ref, _ = orc.render(vol, view, proj, W, H, tf, spv=1.0, value_range=(0.0, 4095.0), mode=mode, iso=1300.0,
                        clip=plane)
    assert_close(img, ref)
    assert not np.array_equal(img, full)


def test_clip_plane_extremes_and_2d(orc, vol_u16):
    sp, vol = vol_u16
    tf = workloads.tf1d_seeded(4096, 11, 900.0, 4095.0)
    view, proj = orbit_camera(35.0, 20.0, 2.5 * workloads.DIAG, 45.0, W, H)
    with _renderer(sp, GBVR_RM_1DTRANS, tf) as r:
        full = _paint(r, view, proj)
        r.setClipPlane((0.0, 0.0, 0.0, 1.0))  # everything on the dropped side
        empty = _paint(r, view, proj)
        assert (empty[..., 3] == 0).all()
        r.setClipPlane((0.0, 0.0, 0.0, -1.0))  # nothing dropped
        assert np.array_equal(_paint(r, view, proj), full)
        r.setClipPlane((0.0, 1.0, 0.0, 0.0), enabled=False)
        assert np.array_equal(_paint(r, view, proj), full)
    tf2 = workloads.tf2d_seeded(256, 128, 5, zero_cols=40)
    plane = (0.6, -0.2, 0.7, 0.0)
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(sp, brick_size=64, overlap=2)
        r.resize((W, H))
        r.setRenderMode(GBVR_RM_2DTRANS)
        r.set2DTrans(tf2, 0.02)
        r.setValueRange(0.0, 4095.0)
        r.setClipPlane(plane)
        img = _paint(r, view, proj)
    ref, _ = orc.render(vol, view, proj, W, H, tf2, spv=1.0, value_range=(0.0, 4095.0), mode=1, grad_max=0.02,
                        clip=plane)
    assert_close(img, ref)


def test_ooc_mip_equals_incore(vol_u16):
    sp, _ = vol_u16
    tf = workloads.tf1d_seeded(4096, 7, 500.0, 4095.0)
    view, proj = orbit_camera(35.0, 20.0, 2.5 * workloads.DIAG, 45.0, W, H)
    with _renderer(sp, GBVR_RM_MIP, tf) as a, Renderer(float_fb=True) as b:
        b.loadSyntheticOutOfCore(sp, 1 << 30, brick_size=64, overlap=2)
        b.resize((W, H))
        b.setRenderMode(GBVR_RM_MIP)
        b.set1DTrans(tf)
        b.setValueRange(0.0, 4095.0)
        b.setSampleRateModifier(1.0)
        assert np.array_equal(_paint(a, view, proj), _paint(b, view, proj))


# ---- 2D slice views ----------------------------------------------------------

@pytest.mark.parametrize("axis", [0, 1, 2])
def test_slices_match_oracle(orc, vol_u16, axis):
    sp, vol = vol_u16
    tf = workloads.tf1d_seeded(4096, 7, 500.0, 4095.0)
    idx = [40, 77, 55][axis]
    with _renderer(sp, GBVR_RM_1DTRANS, tf) as r:
        r.setBGColors((0.2, 0.3, 0.4), (0.2, 0.3, 0.4))
        for flips in [(False, False), (True, False), (False, True)]:
            r.paintSlice(axis, idx, *flips)
            img = r.readFramebuffer(0, as_float=True)
            ref = orc.render_slice(vol, axis, float(idx), W, H, tf, value_range=(0.0, 4095.0), flip_x=flips[0],
                                   flip_y=flips[1], bg=(0.2, 0.3, 0.4))
            assert_close(img, ref)
        assert (ref[..., 3] > 0).mean() > 0.03
        # background outside the letterboxed slice
        assert (img[..., 3] == 0).any()
        r.paintSlice(axis, idx, use_mip=True)
        img = r.readFramebuffer(0, as_float=True)
        samples_skip = r.stats()["samples"]
    ref = orc.render_slice(vol, axis, 0.0, W, H, tf, value_range=(0.0, 4095.0), mip=True, bg=(0.2, 0.3, 0.4))
    assert_close(img, ref)
    # at most one sample per voxel along the axis for each pixel of the slice rectangle
    ext = np.array(DIMS, np.float64) / max(DIMS)
    ua, va = (1, 2) if axis == 0 else ((0, 2) if axis == 1 else (0, 1))
    sc = min(W / ext[ua], H / ext[va])
    assert 0 < samples_skip <= (ext[ua] * sc + 1) * (ext[va] * sc + 1) * DIMS[axis]


def test_slice_lod_and_nearest(orc):
    sp = synth_params((120, 90, 100), np.uint8, 4, 8, (3.0, 9.0), (0.3, 1.0), 255.0, noise_kind=1, noise_amp=4.0,
                      vmax=255.0)
    vol = orc.synth_blobs(sp)
    tf = workloads.tf1d_seeded(256, 4, 30.0, 255.0)
    from imagevis3d_gb300 import GBVR_NEAREST
    with _renderer(sp, GBVR_RM_2DTRANS, tf, rng=(0.0, 255.0)) as r:  # slices use the 1D TF in any mode
        r.set2DTrans(workloads.tf2d_seeded(256, 64, 3), 0.05)
        r.paintSlice(2, 31)
        ref = orc.render_slice(vol, 2, 31.0, W, H, tf, value_range=(0.0, 255.0))
        assert_close(r.readFramebuffer(0, as_float=True), ref)
        # nearest sampling: a canvas size whose pixel centres never land exactly
        # half-way between voxels (there FP32 and FP64 may round either way)
        r.setInterpolant(GBVR_NEAREST)
        r.resize((197, 151))
        r.paintSlice(0, 70)
        ref = orc.render_slice(vol, 0, 70.0, 197, 151, tf, value_range=(0.0, 255.0), interp=0)
        assert_close(r.readFramebuffer(0, as_float=True), ref)
        r.resize((W, H))
        r.setInterpolant(1)
        r.setLODLimits(1, 1)
        r.paintSlice(1, 45)
        # finest-level slice 45 sits at level-1 coordinate (45 + 0.5) * 45 / 90 - 0.5
        ref = orc.render_slice(orc.downsample(vol), 1, (45 + 0.5) * 45 / 90 - 0.5, W, H, tf, value_range=(0.0, 255.0),
                               extent=(1.0, 0.75, 100 / 120))
        assert_close(r.readFramebuffer(0, as_float=True), ref)
        with pytest.raises(Exception):
            r.paintSlice(3, 0)
        with pytest.raises(Exception):
            r.paintSlice(0, 120)
