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
    wl = scene
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(wl.synth, brick_size=64, overlap=2, layouts=4)
        _setup(r, wl)
        r.paintBatch(wl.views)
        one = [r.readFramebuffer(i, as_float=True) for i in range(4)]
        n1 = r.stats()["samples"]
        r.setSamplesPerStep(2)
        r.paintBatch(wl.views)
        two = [r.readFramebuffer(i, as_float=True) for i in range(4)]
        assert r.stats()["samples"] == n1  # the same samples composited
        with pytest.raises(Exception):
            r.setSamplesPerStep(3)
    for a, b in zip(one, two):
        assert np.array_equal(a, b)
    assert max(float(a[..., 3].max()) for a in one) > 0.2


def test_brick_size_rebuild_keeps_pixels_and_histograms(scene):
    wl = scene
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(wl.synth, brick_size=64, overlap=2, layouts=4)
        _setup(r, wl)
        h1 = r.getHistogram()
        h2, mg = r.get2DHistogram()
        r.paintBatch(wl.views)
        ref = [r.readFramebuffer(i, as_float=True) for i in range(4)]
        res = r.autotuneEx(wl.views, brick_sizes=(32, 64, 128), samples_per_step=(1, 2))
        assert res["brick_size"] in (32, 64, 128) and res["samples_per_step"] in (1, 2)
        assert res["candidates"] == 3 * 2 * 12
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
