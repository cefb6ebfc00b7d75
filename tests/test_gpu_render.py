"""Raycaster parity: the CUDA kernels against the FP64 CPU oracle with the
identical sampling rule, within max 2/255 and RMS 0.5/255 per channel."""
import numpy as np
import pytest

from imagevis3d_gb300 import (GBVR_LINEAR, GBVR_NEAREST, GBVR_RM_1DTRANS, GBVR_RM_2DTRANS,
                              GBVR_RM_ISOSURFACE, GBVR_RM_MIP, GBVR_SAMPLER_SW, GBVR_SAMPLER_TEX, GbvrError,
                              Renderer, orbit_camera, synth_params, workloads)
from tests.gpu_util import assert_close

pytestmark = pytest.mark.gpu


def gpu_render(r, view, proj):
    r.setView(view, proj)
    r.paint()
    return r.readFramebuffer(0, as_float=True)


def test_config1_matches_oracle(orc):
    wl = workloads.config1()
    vol = orc.synth_blobs(wl.synth)
    view, proj = wl.views[0]
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(wl.synth, **wl.brick)
        r.resize((wl.width, wl.height))
        r.set1DTrans(wl.tf)
        r.setValueRange(*wl.value_range)
        r.setSampleRateModifier(wl.spv)
        r.setEmptySkipping(0)  # count every sample, as the oracle does
        img = gpu_render(r, view, proj)
        img8 = r.readFramebuffer(0)
        st = r.stats()
    ref, ns = orc.render(vol, view, proj, wl.width, wl.height, wl.tf, spv=wl.spv,
                         value_range=wl.value_range)
    assert_close(img, ref)
    # RGBA8 = round-to-nearest-even of the float32 product c * 255 (saturated)
    want8 = np.rint(np.clip(img, 0, 1).astype(np.float32) * np.float32(255)).astype(np.uint8)
    assert np.array_equal(img8, want8)
    assert (ref[..., 3] > 0.05).mean() > 0.02, "workload renders something"
    # samples counted in-kernel agree with the oracle's count to within ERT/boundary effects
    assert abs(st["samples"] - ns) <= 0.01 * ns


def test_c60_with_reference_tf_matches_oracle(orc, c60):
    vol = c60["volume"]
    tf = c60["tf1d"]
    view, proj = orbit_camera(30.0, 25.0, 2.5 * workloads.DIAG, 45.0, 384, 384)
    with Renderer(float_fb=True) as r:
        r.loadVolume(vol, brick_size=256, overlap=2)
        r.resize((384, 384))
        r.set1DTrans(tf)
        img = gpu_render(r, view, proj)
    ref, _ = orc.render(vol, view, proj, 384, 384, tf, value_range=(0.0, 255.0))
    assert_close(img, ref)
    assert ref[..., 3].max() > 0.5


@pytest.fixture(scope="module")
def multibrick(orc):
    sp = synth_params((150, 130, 110), np.uint16, 11, 10, (4.0, 12.0), (0.3, 1.0), 2600.0,
                      noise_kind=2, noise_amp=20.0, vmax=4095.0, bg_freq=1.0, bg_level=0.15, bg_amp=0.1)
    vol = orc.synth_blobs(sp)
    levels = [vol]
    for _ in orc.lod_dims((150, 130, 110), 64, 2)[1:]:
        levels.append(orc.downsample(levels[-1]))
    tf = workloads.tf1d_seeded(4096, 11, 900.0, 4095.0)
    return vol, levels, tf


@pytest.mark.parametrize("lod", [0, 1, 2])
def test_multibrick_levels_match_oracle(orc, multibrick, lod):
    vol, levels, tf = multibrick
    view, proj = orbit_camera(35.0, 20.0, 2.5 * workloads.DIAG, 45.0, 200, 150)
    with Renderer(float_fb=True) as r:
        r.loadVolume(vol, brick_size=64, overlap=2)
        r.resize((200, 150))
        r.set1DTrans(tf)
        r.setValueRange(0.0, 4095.0)
        r.setSampleRateModifier(1.5)
        r.setLODLimits(lod, 8)
        img = gpu_render(r, view, proj)
        st = r.stats()
    m = max(vol.shape)
    ext = (vol.shape[2] / m, vol.shape[1] / m, vol.shape[0] / m)
    ref, _ = orc.render(levels[lod], view, proj, 200, 150, tf, spv=1.5, value_range=(0.0, 4095.0),
                        extent=ext)
    assert_close(img, ref)
    assert st["lod"] == lod
    if lod == 0:
        assert st["bricks_skipped"] > 0, "the TF leaves background bricks empty"


def test_batch_plain_and_alone_are_bit_identical(multibrick):
    vol, _, tf = multibrick
    views = workloads.orbit_views(5, 120, 96)
    with Renderer(float_fb=True) as r:
        r.loadVolume(vol, brick_size=64, overlap=2)
        r.resize((120, 96))
        r.set1DTrans(tf)
        r.setValueRange(0.0, 4095.0)
        r.setSampleRateModifier(1.5)
        r.paintBatch(views)
        batch = [r.readFramebuffer(i, as_float=True) for i in range(5)]
        sb = r.stats()
        r.paintViews(views)
        plain = [r.readFramebuffer(i, as_float=True) for i in range(5)]
        sp = r.stats()
        # a different mix: reversed order plus a repeat
        r.paintBatch(views[::-1] + views[:2])
        mix = [r.readFramebuffer(i, as_float=True) for i in range(7)]
        alone = []
        for v, p in views:
            r.setView(v, p)
            r.paint()
            alone.append(r.readFramebuffer(0, as_float=True))
    for i in range(5):
        assert np.array_equal(batch[i], plain[i])
        assert np.array_equal(batch[i], alone[i])
        assert np.array_equal(batch[i], mix[4 - i])
    assert np.array_equal(mix[5], batch[0]) and np.array_equal(mix[6], batch[1])
    assert sb["samples"] == sp["samples"] and sb["brick_bytes"] == sp["brick_bytes"]


def test_nearest_interpolant_matches_oracle(orc, multibrick):
    vol, _, tf = multibrick
    view, proj = orbit_camera(200.0, -15.0, 2.5 * workloads.DIAG, 45.0, 160, 120)
    with Renderer(float_fb=True) as r:
        r.loadVolume(vol, brick_size=64, overlap=2)
        r.resize((160, 120))
        r.set1DTrans(tf)
        r.setValueRange(0.0, 4095.0)
        r.setInterpolant(GBVR_NEAREST)
        img = gpu_render(r, view, proj)
    ref, _ = orc.render(vol, view, proj, 160, 120, tf, value_range=(0.0, 4095.0), interp=0)
    assert_close(img, ref)


def test_empty_tf_renders_background_and_skips_everything(multibrick):
    vol, _, _ = multibrick
    tf = np.zeros((256, 4), np.float32)
    tf[:, :3] = 1.0
    with Renderer(float_fb=True) as r:
        r.loadVolume(vol, brick_size=64, overlap=2)
        r.resize((64, 48))
        r.set1DTrans(tf)
        r.setBGColors((0.2, 0.3, 0.4), (0.2, 0.3, 0.4))
        r.paint()
        img = r.readFramebuffer(0, as_float=True)
        st = r.stats()
    assert np.allclose(img[..., :3], [0.2, 0.3, 0.4], atol=1e-7) and np.all(img[..., 3] == 0)
    assert st["bricks_touched"] == 0 and st["samples"] == 0


def test_constant_volume_known_answer(orc):
    vol = np.full((32, 32, 32), 100, np.uint8)
    tf = np.zeros((256, 4), np.float32)
    tf[:, 0] = 1.0
    tf[:, 3] = 0.02
    view, proj = orbit_camera(0.0, 0.0, 3.0, 30.0, 33, 33)
    with Renderer(float_fb=True) as r:
        r.loadVolume(vol, brick_size=32, overlap=2)
        r.resize((33, 33))
        r.set1DTrans(tf)
        img = gpu_render(r, view, proj)
    # the centre ray crosses the unit cube along z: 32 samples of alpha 0.02
    a = 1.0 - (1.0 - 0.02) ** 32
    assert abs(img[16, 16, 3] - a) < 1e-5 and abs(img[16, 16, 0] - a) < 1e-5
    ref, _ = orc.render(vol, view, proj, 33, 33, tf)
    assert_close(img, ref)


def test_2d_tf_with_lighting_matches_oracle(orc, multibrick):
    vol, _, _ = multibrick
    tf2 = workloads.tf2d_seeded(256, 128, 5)
    view, proj = orbit_camera(60.0, 30.0, 2.5 * workloads.DIAG, 45.0, 160, 120)
    with Renderer(float_fb=True) as r:
        r.loadVolume(vol, brick_size=64, overlap=2)
        info = r.datasetInfo()
        gmax = 0.25 * 4095.0 * info["hist2d_max_grad"]
        r.resize((160, 120))
        r.setRenderMode(GBVR_RM_2DTRANS)
        r.set2DTrans(tf2, gmax / 4095.0)
        r.setValueRange(0.0, 4095.0)
        img = gpu_render(r, view, proj)
    ref, _ = orc.render(vol, view, proj, 160, 120, tf2, value_range=(0.0, 4095.0), mode=1,
                        grad_max=gmax / 4095.0)
    assert_close(img, ref)
    assert ref[..., 3].max() > 0.2


@pytest.mark.parametrize("iso", [1000.0, 1300.0, 1600.0])
def test_isosurface_matches_oracle(orc, multibrick, iso):
    vol, _, _ = multibrick
    view, proj = orbit_camera(120.0, 10.0, 2.5 * workloads.DIAG, 45.0, 160, 120)
    with Renderer(float_fb=True) as r:
        r.loadVolume(vol, brick_size=64, overlap=2)
        r.resize((160, 120))
        r.setRenderMode(GBVR_RM_ISOSURFACE)
        r.setIsoValue(iso, (0.9, 0.7, 0.3))
        r.setSampleRateModifier(1.5)
        img = gpu_render(r, view, proj)
    ref, _ = orc.render(vol, view, proj, 160, 120, np.zeros((2, 4), np.float32), spv=1.5, mode=2,
                        iso=iso, iso_rgb=(0.9, 0.7, 0.3), value_range=(0.0, 4095.0))
    hit_g, hit_r = img[..., 3] > 0.5, ref[..., 3] > 0.5
    # first-hit coverage agrees except where a ray grazes the isovalue
    assert (hit_g != hit_r).mean() < 0.002
    both = hit_g & hit_r
    assert_close(img[both], ref[both])
    assert hit_r.mean() > 0.003


def test_relative_isovalue_and_blend_precision(multibrick):
    """setIsoValueRelative(f) renders as setIsoValue(clamp(f, 0, 1) x the
    range top); every blend precision composites the same FP32 image."""
    vol, _, _ = multibrick
    top_value = float(vol.max())  # the range top: the histogram's last non-empty bin
    view, proj = orbit_camera(120.0, 10.0, 2.5 * workloads.DIAG, 45.0, 96, 72)
    with Renderer(float_fb=True) as r:
        r.loadVolume(vol, brick_size=64, overlap=2)
        r.resize((96, 72))
        r.setRenderMode(GBVR_RM_ISOSURFACE)
        r.setIsoValue(float(np.float32(0.3) * np.float32(top_value)))
        absolute = gpu_render(r, view, proj)
        r.setIsoValueRelative(0.3)
        relative = gpu_render(r, view, proj)
        r.setIsoValueRelative(1.7)
        clamped = gpu_render(r, view, proj)
        r.setIsoValue(top_value)
        top = gpu_render(r, view, proj)
        for bits in (8, 16, 32):
            r.setBlendPrecision(bits)
            assert np.array_equal(gpu_render(r, view, proj), top)
        with pytest.raises(GbvrError):
            r.setBlendPrecision(12)
    assert np.array_equal(relative, absolute)
    assert np.array_equal(clamped, top)
    assert (absolute[..., 3] > 0.5).mean() > 0.003


def test_texture_sampler_matches_oracle(orc, multibrick):
    vol, _, tf = multibrick
    view, proj = orbit_camera(35.0, 20.0, 2.5 * workloads.DIAG, 45.0, 200, 150)
    with Renderer(float_fb=True) as r:
        r.loadVolume(vol, brick_size=64, overlap=2, build_texture=True)
        r.resize((200, 150))
        r.set1DTrans(tf)
        r.setValueRange(0.0, 4095.0)
        r.setSampleRateModifier(1.5)
        r.setSampler(GBVR_SAMPLER_TEX)
        img_tex = gpu_render(r, view, proj)
        r.setSampler(GBVR_SAMPLER_SW)
        img_sw = gpu_render(r, view, proj)
    ref, _ = orc.render(vol, view, proj, 200, 150, tf, spv=1.5, value_range=(0.0, 4095.0))
    assert_close(img_sw, ref)
    assert_close(img_tex, ref)


def test_state_errors_are_statuses():
    with Renderer() as r:
        with pytest.raises(GbvrError) as e:
            r.paint()
        assert e.value.code == -7
        with pytest.raises(GbvrError):
            r.setSampleRateModifier(0.0)
        with pytest.raises(GbvrError):
            r.resize((0, 10))
        with pytest.raises(GbvrError):
            r.loadDataset("/nonexistent.uvf")


def test_layout_copies_and_launch_shapes_do_not_change_pixels(multibrick):
    """x/y/z-fastest brick copies and every warp tile shape give the same
    image bit for bit: only the memory order and the schedule change."""
    vol, _, tf = multibrick
    views = workloads.orbit_views(4, 96, 80, elevation=35.0, start=10.0)
    views.append(orbit_camera(0.0, 89.0, 2.5 * workloads.DIAG, 45.0, 96, 80))  # looking down y
    imgs = {}
    for layouts in (1, 3, 4, 5, 6):
        with Renderer(float_fb=True) as r:
            r.loadVolume(vol, brick_size=64, overlap=2, layouts=layouts)
            r.resize((96, 80))
            r.set1DTrans(tf)
            r.setValueRange(0.0, 4095.0)
            r.setSampleRateModifier(1.5)
            for tw in ((8, 16, 32, 4) if layouts == 3 else (8, 4)):
                r.setLaunchShape(tw, 0)
                r.paintBatch(views)
                imgs[(layouts, tw)] = [r.readFramebuffer(i, as_float=True) for i in range(len(views))]
            if layouts == 3:
                tune = r.autotune(views)
                assert tune["tile_w"] in (4, 8, 16, 32) and tune["candidates"] == 12
                assert tune["best_ms"] <= tune["default_ms"]
                r.paintBatch(views)
                imgs["tuned"] = [r.readFramebuffer(i, as_float=True) for i in range(len(views))]
    ref = imgs[(1, 8)]
    for key, got in imgs.items():
        for i in range(len(views)):
            assert np.array_equal(got[i], ref[i]), (key, i)


@pytest.mark.parametrize("mode", [GBVR_RM_1DTRANS, GBVR_RM_2DTRANS, GBVR_RM_ISOSURFACE, GBVR_RM_MIP])
@pytest.mark.parametrize("interp", [True, False])
def test_overlapped_blocks_give_the_same_pixels(multibrick, mode, interp):
    """The copy in 4^3 blocks that hold their +1 neighbours (layouts 5, and 6
    where isosurfaces use it) reads the same voxels as the x-fastest copy in
    every mode, with trilinear and nearest sampling: the same pixels bit for
    bit."""
    vol, _, tf = multibrick
    views = workloads.orbit_views(3, 112, 96, elevation=25.0, start=40.0)
    out = {}
    for layouts in (1, 5, 6):
        with Renderer(float_fb=True) as r:
            r.loadVolume(vol, brick_size=64, overlap=2, layouts=layouts)
            r.resize((112, 96))
            r.set1DTrans(tf)
            r.setValueRange(0.0, 4095.0)
            r.setSampleRateModifier(1.5)
            r.setInterpolant(GBVR_LINEAR if interp else GBVR_NEAREST)
            r.setRenderMode(mode)
            if mode == GBVR_RM_2DTRANS:
                r.set2DTrans(workloads.tf2d_seeded(256, 64, 5, widgets=3), r.datasetInfo()["hist2d_max_grad"])
            if mode == GBVR_RM_ISOSURFACE:
                r.setIsoValue(1500.0, (0.8, 0.8, 0.9))
            r.paintBatch(views)
            out[layouts] = [r.readFramebuffer(i, as_float=True) for i in range(len(views))]
    assert max(float(a[..., 3].max()) for a in out[1]) > 0.2
    for lay in (5, 6):
        for a, b in zip(out[1], out[lay]):
            assert np.array_equal(a, b), lay


@pytest.mark.parametrize("mode", [GBVR_RM_1DTRANS, GBVR_RM_2DTRANS, GBVR_RM_ISOSURFACE])
def test_empty_space_skipping_is_exact(multibrick, mode):
    """No skipping, brick skipping and macro-cell skipping give the same bits."""
    vol, _, tf = multibrick
    views = workloads.orbit_views(3, 128, 96, elevation=25.0, start=15.0)
    out = []
    for skip in (0, 1, 2):
        with Renderer(float_fb=True) as r:
            r.loadVolume(vol, brick_size=64, overlap=2)
            r.resize((128, 96))
            r.setRenderMode(mode)
            if mode == GBVR_RM_2DTRANS:
                r.set2DTrans(workloads.tf2d_seeded(256, 64, 9), 0.05)
            elif mode == GBVR_RM_ISOSURFACE:
                r.setIsoValue(1300.0, (1.0, 0.8, 0.5))
            else:
                r.set1DTrans(tf)
            r.setValueRange(0.0, 4095.0)
            r.setSampleRateModifier(1.5)
            r.setEmptySkipping(skip)
            r.paintBatch(views)
            out.append(([r.readFramebuffer(i, as_float=True) for i in range(3)], r.stats()))
    for i in range(3):
        assert np.array_equal(out[0][0][i], out[1][0][i])
        assert np.array_equal(out[0][0][i], out[2][0][i])
    if mode != GBVR_RM_ISOSURFACE:
        # skipping removes samples, never adds
        assert out[2][1]["samples"] <= out[1][1]["samples"] <= out[0][1]["samples"]
    if mode == GBVR_RM_1DTRANS:
        assert out[2][1]["samples"] < out[0][1]["samples"]


def test_batch_readback_matches_per_view_readback(multibrick):
    vol, _, tf = multibrick
    views = workloads.orbit_views(3, 64, 40)
    with Renderer() as r:
        r.loadVolume(vol, brick_size=64, overlap=2)
        r.resize((64, 40))
        r.set1DTrans(tf)
        r.paintBatch(views)
        allv = r.readFramebuffers()
        assert allv.shape == (3, 40, 64, 4)
        for i in range(3):
            assert np.array_equal(allv[i], r.readFramebuffer(i))
        assert np.array_equal(r.readFramebuffers(1, 2)[1], allv[2])
        with pytest.raises(GbvrError):
            r.readFramebuffers(2, 2)
