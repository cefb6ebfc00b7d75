"""Autotuner dimensions: launch shape, brick size (the dataset rebuilt from
its finest level) and samples per inner-loop step.  None of them changes a
pixel; the tuner keeps its fastest combination set."""
import numpy as np
import pytest

from imagevis3d_gb300 import GBVR_RM_ISOSURFACE, Renderer, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    wl = workloads.config2(size=192, width=160, height=120, nviews=4)
    wl.views = workloads.orbit_views(4, 160, 120, radius=1.6 * workloads.DIAG, start=10.0)
    return wl


def _setup(r, wl):
    r.resize((wl.width, wl.height))
    r.set1DTrans(wl.tf)
    r.setValueRange(*wl.value_range)
    r.setSampleRateModifier(wl.spv)


def test_samples_per_step_keeps_the_pixels(scene):
    """1 (one sample per lane per step), 2 (two in flight per lane), 4 and 8
    (the warp evaluates the pending samples of all its rays together): the
    same samples composited in the same order, so the same pixels and sample
    counts -- also with a clip plane, with each empty-space skipping mode and in
    the stats pass that records the sampled macro-cells."""
    wl = scene
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(wl.synth, brick_size=64, overlap=2, layouts=4)
        _setup(r, wl)

        def frames():
            r.paintBatch(wl.views)
            st = r.stats()
            return [r.readFramebuffer(i, as_float=True) for i in range(4)], st["samples"], st["cells_touched"]

        for clip in (None, (0.3, -0.5, 0.8, 0.05)):
            if clip is not None:
                r.setClipPlane(clip)
            for skip in (2, 1, 0):
                r.setEmptySkipping(skip)
                for level in (1, 2):
                    r.setStatsLevel(level)
                    r.setSamplesPerStep(1)
                    ref, n1, c1 = frames()
                    for sps in (2, 4, 8):
                        r.setSamplesPerStep(sps)
                        got, n, c = frames()
                        assert n == n1 and c == c1, (clip, skip, level, sps)
                        for a, b in zip(ref, got):
                            assert np.array_equal(a, b), (clip, skip, level, sps)
            assert max(float(a[..., 3].max()) for a in ref) > 0.2
        with pytest.raises(Exception):
            r.setSamplesPerStep(3)


def test_brick_size_rebuild_keeps_pixels_and_histograms(scene):
    wl = scene
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(wl.synth, brick_size=64, overlap=2, layouts=4)
        _setup(r, wl)
        h1 = r.getHistogram()
        h2, mg = r.get2DHistogram()
        r.paintBatch(wl.views)
        ref = [r.readFramebuffer(i, as_float=True) for i in range(4)]
        res = r.autotuneEx(wl.views, brick_sizes=(32, 64, 128), samples_per_step=(1, 2, 4, 8))
        assert res["brick_size"] in (32, 64, 128) and res["samples_per_step"] in (1, 2, 4, 8)
        assert res["candidates"] == 3 * 4 * 12
        assert 0 < res["best_ms"] <= res["default_ms"] <= res["worst_ms"]
        info = r.datasetInfo()
        assert info["brick_size"] == res["brick_size"]
        assert np.array_equal(r.getHistogram(), h1)
        g2, gmg = r.get2DHistogram()
        assert np.array_equal(g2, h2) and np.float32(gmg) == np.float32(mg)
        r.paintBatch(wl.views)
        for i in range(4):
            assert np.array_equal(r.readFramebuffer(i, as_float=True), ref[i]), i
        # other modes after the rebuild: isosurface at each brick size equals the 64 build
        r.setRenderMode(GBVR_RM_ISOSURFACE)
        r.setIsoValue(2000.0, (0.8, 0.8, 0.9))
        r.paintBatch(wl.views)
        iso = [r.readFramebuffer(i, as_float=True) for i in range(4)]
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(wl.synth, brick_size=64, overlap=2, layouts=4)
        _setup(r, wl)
        r.setRenderMode(GBVR_RM_ISOSURFACE)
        r.setIsoValue(2000.0, (0.8, 0.8, 0.9))
        r.paintBatch(wl.views)
        for i in range(4):
            assert np.array_equal(r.readFramebuffer(i, as_float=True), iso[i]), i
