"""Out-of-core datasets (bricks in page-locked host memory, a device slot pool
with LRU residency, LOD fallback on overflow).

The streaming build must store the same bricks, brick ranges and histogram as
the in-core build of the same seeded volume; a paint that resolves level l
must give the image the in-core renderer gives at level l, bit for bit (the
skipped bricks are empty under the TF or outside every view frustum, where no
ray samples); and with the eye inside the volume the image must match the FP64
oracle within the raycaster's tolerance."""
import numpy as np
import pytest

from imagevis3d_gb300 import (GBVR_RM_1DTRANS, GBVR_RM_ISOSURFACE, GBVR_SAMPLER_TEX, GbvrError, Renderer,
                              orbit_camera, synth_params, workloads)
from tests.gpu_util import assert_close

pytestmark = pytest.mark.gpu

CASES = {
    "u16_200x180x170_b64": (synth_params((200, 180, 170), np.uint16, 21, 12, (5.0, 14.0), (0.3, 1.0), 2600.0,
                                         noise_kind=2, noise_amp=20.0, vmax=4095.0, bg_freq=1.0, bg_level=0.1,
                                         bg_amp=0.1), dict(brick_size=64, overlap=2)),
    "u8_131x97x203_b32": (synth_params((131, 97, 203), np.uint8, 5, 9, (3.0, 9.0), (0.3, 1.0), 255.0,
                                       noise_kind=1, noise_amp=4.0, vmax=255.0), dict(brick_size=32, overlap=2)),
    "f32_90x75x140_b32_ov3": (synth_params((90, 75, 140), np.float32, 8, 6, (3.0, 8.0), (0.3, 1.0), 1.0,
                                           noise_kind=2, noise_amp=0.01, vmax=0.0),
                              dict(brick_size=32, overlap=3)),
}
BIG_POOL = 1 << 30


def _tf(sp):
    if sp.dtype == 1:
        return workloads.tf1d_seeded(4096, 21, 900.0, 4095.0), (0.0, 4095.0)
    if sp.dtype == 0:
        return workloads.tf1d_seeded(256, 5, 40.0, 255.0), (0.0, 255.0)
    return workloads.tf1d_seeded(256, 8, 0.15, 1.0), (0.0, 1.0)


def _setup(r, sp, w, h):
    tf, rng = _tf(sp)
    r.resize((w, h))
    r.set1DTrans(tf)
    r.setValueRange(*rng)
    r.setSampleRateModifier(1.0)


def _paint(r, view, proj):
    r.setView(view, proj)
    r.paint()
    return r.readFramebuffer(0, as_float=True)


@pytest.mark.parametrize("case", sorted(CASES))
def test_ooc_build_matches_incore(case):
    sp, bp = CASES[case]
    with Renderer() as a, Renderer() as b:
        a.loadSynthetic(sp, **bp)
        b.loadSyntheticOutOfCore(sp, BIG_POOL, **bp)
        ia, ib = a.datasetInfo(), b.datasetInfo()
        for k in ("dims", "lod_count", "lod_dims", "lod_bricks", "total_bricks", "range", "hist1d_size"):
            assert ia[k] == ib[k], k
        assert ib["host_bytes"] > 0 and ib["device_slots"] == ib["total_bricks"]
        if sp.dtype != 2:
            assert np.array_equal(a.getHistogram(), b.getHistogram())
            # the 2D histogram, streamed in z-slabs out of core, bit for bit
            h2a, ga = a.get2DHistogram()
            h2b, gb = b.get2DHistogram()
            assert ga == gb > 0 and np.array_equal(h2a, h2b)
            assert ia["hist2d_max_grad"] == ib["hist2d_max_grad"]
        for lod in range(ia["lod_count"]):
            assert np.array_equal(a.brickMinMax(lod), b.brickMinMax(lod))
            nb = ia["lod_bricks"][lod]
            for bz in range(nb[2]):
                for by in range(nb[1]):
                    for bx in range(nb[0]):
                        va, oa = a.getBrick(lod, (bx, by, bz))
                        vb, ob = b.getBrick(lod, (bx, by, bz))
                        assert oa == ob and np.array_equal(va, vb), (lod, bx, by, bz)


def test_ooc_bricks_match_oracle(orc):
    sp, bp = CASES["u8_131x97x203_b32"]
    vol = orc.synth_blobs(sp)
    with Renderer() as r:
        r.loadSyntheticOutOfCore(sp, 64 * 32 ** 3, **bp)
        info = r.datasetInfo()
        assert info["device_slots"] == 64
        level = vol
        for lod in range(info["lod_count"]):
            if lod:
                level = orc.downsample(level)
            nb = info["lod_bricks"][lod]
            for b in [(0, 0, 0), (nb[0] - 1, nb[1] - 1, nb[2] - 1), (nb[0] // 2, 0, nb[2] // 2)]:
                want, wo = orc.extract_brick(level, bp["brick_size"], bp["overlap"], b)
                got, go = r.getBrick(lod, b)
                assert go == wo and np.array_equal(got, want), (lod, b)


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("mode", [GBVR_RM_1DTRANS, GBVR_RM_ISOSURFACE])
def test_ooc_render_equals_incore(case, mode):
    sp, bp = CASES[case]
    views = [orbit_camera(az, el, 2.5 * workloads.DIAG, 45.0, 160, 120) for az, el in ((20, 15), (140, -30), (260, 50))]
    _, rng = _tf(sp)
    iso = rng[0] + 0.3 * (rng[1] - rng[0])
    with Renderer(float_fb=True) as a, Renderer(float_fb=True) as b:
        a.loadSynthetic(sp, **bp)
        b.loadSyntheticOutOfCore(sp, BIG_POOL, **bp)
        for r in (a, b):
            _setup(r, sp, 160, 120)
            r.setRenderMode(mode)
            r.setIsoValue(iso)
        for view, proj in views:
            ia = _paint(a, view, proj)
            ib = _paint(b, view, proj)
            st = b.stats()
            assert st["lod"] == 0
            assert np.array_equal(ia, ib)
        assert ia[..., 3].max() > 0.3
        b.paintBatch(views)
        for i, (view, proj) in enumerate(views):
            assert np.array_equal(b.readFramebuffer(i, as_float=True), _paint(a, view, proj))


def test_ooc_small_pool_falls_back_to_coarser_level():
    sp, bp = CASES["u16_200x180x170_b64"]
    slot = 64 ** 3 * 2
    view, proj = orbit_camera(35.0, 20.0, 2.5 * workloads.DIAG, 45.0, 200, 150)
    with Renderer(float_fb=True) as a, Renderer(float_fb=True) as b:
        a.loadSynthetic(sp, **bp)
        b.loadSyntheticOutOfCore(sp, 6 * slot, **bp)
        assert b.datasetInfo()["device_slots"] == 6
        _setup(a, sp, 200, 150)
        _setup(b, sp, 200, 150)
        img = _paint(b, view, proj)
        st = b.stats()
        assert st["lod"] > 0
        assert st["brick_misses"] > 0 and st["bytes_paged"] > 0
        a.setLODLimits(st["lod"], st["lod"])
        assert np.array_equal(img, _paint(a, view, proj))
        # the same frame again: everything resident, nothing paged
        _paint(b, view, proj)
        assert b.stats()["bytes_paged"] == 0


def _inside_path(frames, w, h):
    keys = [((-0.35, 0.05, -0.3), (0.2, 0.0, 0.1), (0, 1, 0)),
            ((-0.1, 0.0, -0.2), (0.3, 0.0, 0.2), (0, 1, 0)),
            ((0.15, -0.05, 0.0), (0.0, 0.0, 0.35), (0, 1, 0)),
            ((0.1, 0.05, 0.25), (-0.3, 0.0, 0.1), (0, 1, 0))]
    return workloads.flythrough_views(keys, frames, w, h, fov=60.0)


def test_ooc_flythrough_pages_reuses_and_matches_incore():
    sp, bp = CASES["u16_200x180x170_b64"]
    slot = 64 ** 3 * 2
    views = _inside_path(8, 128, 96)
    with Renderer(float_fb=True) as a, Renderer(float_fb=True) as b:
        a.loadSynthetic(sp, **bp)
        b.loadSyntheticOutOfCore(sp, 30 * slot, **bp)
        _setup(a, sp, 128, 96)
        _setup(b, sp, 128, 96)
        paged = []
        for view, proj in views:
            img = _paint(b, view, proj)
            st = b.stats()
            a.setLODLimits(st["lod"], st["lod"])
            assert np.array_equal(img, _paint(a, view, proj))
            paged.append(st["bytes_paged"])
        assert paged[0] > 0
        # consecutive frames share most of their bricks
        assert sum(paged[1:]) < len(paged[1:]) * paged[0]


def test_ooc_eye_inside_matches_oracle(orc):
    sp, bp = CASES["u16_200x180x170_b64"]
    vol = orc.synth_blobs(sp)
    tf, rng = _tf(sp)
    view, proj = _inside_path(3, 128, 96)[1]
    with Renderer(float_fb=True) as r:
        r.loadSyntheticOutOfCore(sp, BIG_POOL, **bp)
        _setup(r, sp, 128, 96)
        img = _paint(r, view, proj)
        assert r.stats()["lod"] == 0
    ref, _ = orc.render(vol, view, proj, 128, 96, tf, spv=1.0, value_range=rng)
    assert_close(img, ref)
    assert ref[..., 3].max() > 0.3


def test_ooc_rejections(tmp_path):
    sp, bp = CASES["u8_131x97x203_b32"]
    with Renderer() as r:
        with pytest.raises(GbvrError):
            r.loadSyntheticOutOfCore(sp, 1000, **bp)  # smaller than one brick
        r.loadSyntheticOutOfCore(sp, BIG_POOL, **bp)
        with pytest.raises(GbvrError):
            r.writeUVF(str(tmp_path / "x.uvf"))
        with pytest.raises(GbvrError):
            r.setSampler(GBVR_SAMPLER_TEX)
            r.paint()



def test_ooc_paint_path_pipeline_matches_incore_per_frame():
    sp, bp = CASES["u16_200x180x170_b64"]
    slot = 64 ** 3 * 2
    views = _inside_path(10, 128, 96)
    with Renderer(float_fb=True) as a, Renderer(float_fb=True) as b, Renderer(float_fb=True) as c:
        a.loadSynthetic(sp, **bp)
        b.loadSyntheticOutOfCore(sp, 30 * slot, **bp)
        c.loadSyntheticOutOfCore(sp, 30 * slot, **bp)
        for r in (a, b, c):
            _setup(r, sp, 128, 96)
        lod, miss, paged = b.paintPath(views)
        st = b.stats()
        assert st["bytes_paged"] == int(paged.sum()) > 0 and st["brick_misses"] == int(miss.sum())
        frames = [b.readFramebuffer(i, as_float=True) for i in range(len(views))]
        for i, (view, proj) in enumerate(views):
            # same level as a synchronous paint of the frame
            img_c = _paint(c, view, proj)
            assert c.stats()["lod"] == lod[i]
            assert np.array_equal(frames[i], img_c), i
            a.setLODLimits(int(lod[i]), int(lod[i]))
            assert np.array_equal(frames[i], _paint(a, view, proj)), i
        # a second pass over the same path finds most bricks resident
        lod2, miss2, paged2 = b.paintPath(views)
        assert paged2.sum() < paged.sum()
        assert np.array_equal(lod2, lod)


def test_path_capture_equals_read_back_frames():
    """gbvr_paint_path_capture: each frame's RGBA8 pixels, copied out while
    later frames page and render, equal the frames read back after a plain
    path paint (out of core, a small pool that pages every frame; and in
    core); a buffer one frame short is rejected."""
    import torch
    sp, bp = CASES["u16_200x180x170_b64"]
    slot = 64 ** 3 * 2
    views = _inside_path(10, 128, 96)
    with Renderer() as b, Renderer() as a:
        b.loadSyntheticOutOfCore(sp, 30 * slot, **bp)
        a.loadSynthetic(sp, **bp)
        for r in (a, b):
            _setup(r, sp, 128, 96)
            lod, miss, paged = r.paintPath(views)
            want = r.readFramebuffers(0, len(views))
            cap = torch.zeros((len(views), 96, 128, 4), dtype=torch.uint8).pin_memory()
            lod2, miss2, paged2 = r.paintPath(views, capture=cap)
            assert np.array_equal(cap.numpy(), want) and np.array_equal(lod2, lod)
            assert np.array_equal(r.readFramebuffers(0, len(views)), want)
        short = np.zeros((len(views) - 1, 96, 128, 4), np.uint8)
        with pytest.raises(GbvrError) as e:
            b.paintPath(views, capture=short)
        assert e.value.code == -1


def test_paint_path_in_core_equals_views():
    sp, bp = CASES["u8_131x97x203_b32"]
    views = _inside_path(4, 96, 64)
    with Renderer(float_fb=True) as a:
        a.loadSynthetic(sp, **bp)
        _setup(a, sp, 96, 64)
        lod, miss, paged = a.paintPath(views)
        assert (lod == 0).all() and miss.sum() == 0 and paged.sum() == 0
        got = [a.readFramebuffer(i, as_float=True) for i in range(4)]
        for i, (view, proj) in enumerate(views):
            assert np.array_equal(got[i], _paint(a, view, proj))


def test_ooc_paint_path_with_bboxes_matches_incore():
    """Bounding-box lines on the pipelined out-of-core path: each frame equals
    the in-core render at its resolved level with the same lines (the brick
    grid of that level)."""
    sp, bp = CASES["u16_200x180x170_b64"]
    slot = 64 ** 3 * 2
    views = _inside_path(6, 128, 96)
    with Renderer(float_fb=True) as a, Renderer(float_fb=True) as b:
        a.loadSynthetic(sp, **bp)
        b.loadSyntheticOutOfCore(sp, 30 * slot, **bp)
        for r in (a, b):
            _setup(r, sp, 128, 96)
            r.setGlobalBBox(True)
            r.setLocalBBox(True, (0.2, 0.8, 0.4))
        lod, _, _ = b.paintPath(views)
        frames = [b.readFramebuffer(i, as_float=True) for i in range(len(views))]
        for i, (view, proj) in enumerate(views):
            a.setLODLimits(int(lod[i]), int(lod[i]))
            assert np.array_equal(frames[i], _paint(a, view, proj)), i
        assert any((f[..., 3] == 1.0).sum() > 50 for f in frames)


@pytest.mark.parametrize("mip", [False, True])
def test_ooc_slices_equal_incore(mip):
    """2D slices of an out-of-core dataset page in the slice's bricks (every
    brick for slice MIP, on a coarser level when they do not fit) and equal
    the in-core slice at that level bit for bit."""
    sp, bp = CASES["u8_131x97x203_b32"]
    slot = 32 ** 3
    with Renderer(float_fb=True) as a, Renderer(float_fb=True) as b:
        a.loadSynthetic(sp, **bp)
        b.loadSyntheticOutOfCore(sp, 48 * slot, **bp)
        for r in (a, b):
            _setup(r, sp, 160, 120)
        lods, visible = set(), 0
        # a sparse TF (empty bricks are skipped) and a dense one
        ramp = np.linspace(0.0, 1.0, 256, dtype=np.float32)
        dense = np.stack([ramp, ramp[::-1], np.full(256, 0.5, np.float32), np.full(256, 0.6, np.float32)], -1)
        dense[0, 3] = 0.0
        for tf in (workloads.tf1d_seeded(256, 5, 40.0, 255.0), dense):
            for r in (a, b):
                r.set1DTrans(tf)
            for axis, idx, fx in ((0, 5, False), (1, 48, True), (2, 150, False), (2, 0, False), (0, 130, True)):
                b.paintSlice(axis, idx, flip_x=fx, use_mip=mip)
                got = b.readFramebuffer(0, as_float=True)
                lod = b.stats()["lod"]
                lods.add(lod)
                a.setLODLimits(lod, lod)
                a.paintSlice(axis, idx, flip_x=fx, use_mip=mip)
                assert np.array_equal(got, a.readFramebuffer(0, as_float=True)), (axis, idx)
                visible += int((got[..., 3] > 0).sum())
        assert visible > 20000
        # slice MIP needs all 160 bricks of level 0: it falls back; a slice fits
        assert lods == ({1} if mip else {0})


@pytest.mark.parametrize("codec", [3, 1], ids=["lz4", "zlib"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_ooc_compressed_store_equals_raw_store(case, codec):
    """The compressed host store (LZ4, codec id 3, or zlib, codec id 1) holds
    the same bricks (decoded on the host) and pages the same bricks (decoded on
    the GPU): images of a paged fly-through equal the raw store's bit for bit."""
    sp, bp = CASES[case]
    slot = (bp["brick_size"] ** 3) * (1 if sp.dtype == 0 else 2 if sp.dtype == 1 else 4)
    views = _inside_path(6, 128, 96)
    with Renderer(float_fb=True) as a, Renderer(float_fb=True) as b:
        a.loadSyntheticOutOfCore(sp, 30 * slot, **bp)
        b.loadSyntheticOutOfCore(sp, 30 * slot, compression=codec, **bp)
        ia, ib = a.datasetInfo(), b.datasetInfo()
        assert ib["compression"] == codec and ib["host_raw_bytes"] == ia["host_bytes"] > 0
        assert 0 < ib["host_bytes"] <= ib["host_raw_bytes"] * 1.01
        for lod in range(ia["lod_count"]):
            nb = ia["lod_bricks"][lod]
            for bz in range(nb[2]):
                for by in range(nb[1]):
                    for bx in range(nb[0]):
                        va, oa = a.getBrick(lod, (bx, by, bz))
                        vb, ob = b.getBrick(lod, (bx, by, bz))
                        assert oa == ob and np.array_equal(va, vb), (lod, bx, by, bz)
        for r in (a, b):
            _setup(r, sp, 128, 96)
        la, _, pa = a.paintPath(views)
        lb, _, pb = b.paintPath(views)
        assert np.array_equal(la, lb) and np.array_equal(pa, pb)
        st = b.stats()
        assert st["bytes_paged_compressed"] > 0
        for i in range(len(views)):
            assert np.array_equal(a.readFramebuffer(i, as_float=True), b.readFramebuffer(i, as_float=True)), i
        # synchronous paints and a slice page through the same decoder
        a.setView(*views[3])
        b.setView(*views[3])
        a.paint()
        b.paint()
        assert np.array_equal(a.readFramebuffer(0, as_float=True), b.readFramebuffer(0, as_float=True))
        a.paintSlice(2, 40)
        b.paintSlice(2, 40)
        assert np.array_equal(a.readFramebuffer(0, as_float=True), b.readFramebuffer(0, as_float=True))


@pytest.mark.parametrize("codec", [3, 1], ids=["lz4", "zlib"])
def test_ooc_compression_shrinks_smooth_volumes(codec):
    sp = synth_params((192, 160, 144), np.uint8, 33, 10, (10.0, 30.0), (0.4, 1.0), 255.0, vmax=255.0,
                      bg_freq=1.0, bg_level=0.1, bg_amp=0.1)
    with Renderer() as r:
        r.loadSyntheticOutOfCore(sp, 1 << 28, brick_size=64, overlap=2, compression=codec)
        info = r.datasetInfo()
    assert info["host_bytes"] * 2 < info["host_raw_bytes"]


@pytest.mark.parametrize("order", [1, 2, 3], ids=["morton", "hilbert", "random"])
@pytest.mark.parametrize("codec", [0, 3], ids=["raw", "lz4"])
def test_ooc_store_orders_page_the_same_bricks(order, codec):
    """Every host-store brick order (the converter's brick layouts: Morton,
    Hilbert, random) holds and pages the same bricks as the scanline order:
    a fly-through gives the same images bit for bit, raw or compressed, and
    each paint's host-to-device copies are counted (one per stretch of bricks
    adjacent in the store)."""
    sp, bp = CASES["u16_200x180x170_b64"]
    slot = (bp["brick_size"] ** 3) * 2
    views = _inside_path(6, 128, 96)
    with Renderer(float_fb=True) as a, Renderer(float_fb=True) as b:
        a.loadSyntheticOutOfCore(sp, 30 * slot, compression=codec, **bp)
        b.loadSyntheticOutOfCore(sp, 30 * slot, compression=codec, brick_order=order, **bp)
        ia, ib = a.datasetInfo(), b.datasetInfo()
        assert ia["host_bytes"] == ib["host_bytes"] > 0
        for lod in range(ia["lod_count"]):
            nb = ia["lod_bricks"][lod]
            for k in range(0, nb[0] * nb[1] * nb[2], 3):
                bx, by, bz = k % nb[0], (k // nb[0]) % nb[1], k // (nb[0] * nb[1])
                va, oa = a.getBrick(lod, (bx, by, bz))
                vb, ob = b.getBrick(lod, (bx, by, bz))
                assert oa == ob and np.array_equal(va, vb), (lod, bx, by, bz)
        for r in (a, b):
            _setup(r, sp, 128, 96)
        la, _, pa = a.paintPath(views)
        lb, _, pb = b.paintPath(views)
        assert np.array_equal(la, lb) and np.array_equal(pa, pb)
        for i in range(len(views)):
            assert np.array_equal(a.readFramebuffer(i, as_float=True), b.readFramebuffer(i, as_float=True)), i
        a.setView(*views[2])
        b.setView(*views[2])
        a.paint()
        b.paint()
        assert np.array_equal(a.readFramebuffer(0, as_float=True), b.readFramebuffer(0, as_float=True))
        sa, sb = a.stats(), b.stats()
        assert sa["brick_misses"] == sb["brick_misses"] and sa["bytes_paged"] == sb["bytes_paged"]
        for st in (sa, sb):
            assert (st["host_copies"] > 0) == (st["bytes_paged"] > 0)
