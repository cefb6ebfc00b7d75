"""Error paths of the renderer's loads, reached without any GPU fault: an
allocation larger than the device (a plain failed cudaMalloc), a failed
page-locked allocation (host-side failure injection), a brick above the
device limit (the reference rebricks a dataset whose bricks exceed the
texture limit: DSBricksOversized, ImageVis3D/UI/ImageVis3D_FileHandling.cpp:
646-690).  After each failure the renderer still loads and paints."""
import numpy as np
import pytest

from imagevis3d_gb300 import GbvrError, Renderer, synth_params, workloads

pytestmark = pytest.mark.gpu

ENOMEM, EOVERSIZED, ESTATE = -3, -8, -7


def _paints(r):
    wl = workloads.config1()
    r.loadSynthetic(wl.synth, **wl.brick)
    r.resize((64, 64))
    r.set1DTrans(wl.tf)
    r.setValueRange(*wl.value_range)
    r.setView(*wl.views[0])
    r.paint()
    assert r.readFramebuffer(0)[..., 3].max() > 0


def test_volume_larger_than_the_device_is_enomem():
    # 8192 x 8192 x 8192 uint8 = 512 GiB: more than any GB300 holds
    p = synth_params((8192, 8192, 8192), np.uint8, 1, 4, (50.0, 90.0), (0.3, 1.0), 255.0)
    with Renderer() as r:
        with pytest.raises(GbvrError) as e:
            r.loadSynthetic(p, brick_size=256, overlap=2)
        assert e.value.code == ENOMEM
        with pytest.raises(GbvrError) as e:
            r.paint()
        assert e.value.code == ESTATE  # nothing loaded
        _paints(r)


def test_failed_page_locked_allocation_is_enomem(monkeypatch):
    wl = workloads.config1()
    with Renderer() as r:
        monkeypatch.setenv("GBVR_FAULT_INJECT", "pinned_alloc")
        with pytest.raises(GbvrError) as e:
            r.loadSyntheticOutOfCore(wl.synth, 1 << 24, brick_size=64, overlap=2)
        assert e.value.code == ENOMEM and "page-locked" in str(e.value)
        monkeypatch.delenv("GBVR_FAULT_INJECT")
        r.loadSyntheticOutOfCore(wl.synth, 1 << 24, brick_size=64, overlap=2)
        _paints(r)


def test_brick_above_the_device_limit_is_eoversized():
    wl = workloads.config1()
    with Renderer() as r:
        with pytest.raises(GbvrError) as e:
            r.loadSynthetic(wl.synth, brick_size=4096, overlap=2)
        assert e.value.code == EOVERSIZED and "2048" in str(e.value)
        _paints(r)
