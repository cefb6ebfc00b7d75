"""The sparse fractal workload (2D transfer function + Phong, isosurfaces,
GPU 2D histogram): generator bit-exact against the CPU restatement, renders
within tolerance of the FP64 oracle, and the UVF build bit-exact."""
import numpy as np
import pytest

from imagevis3d_gb300 import (GBVR_RM_2DTRANS, GBVR_RM_ISOSURFACE, Renderer, fbm_params, fbm_volume,
                              orbit_camera, workloads)
from tests.gpu_util import assert_close

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,dtype", [((64, 64, 64), np.uint8), ((50, 40, 30), np.uint16),
                                        ((33, 47, 21), np.float32)])
def test_fbm_generator_bit_exact(orc, dims, dtype):
    p = fbm_params(dims, dtype, 99, octaves=6, base_period=2, threshold=0.5,
                   vmax=255.0 if dtype == np.uint8 else 4095.0)
    assert np.array_equal(fbm_volume(p), orc.synth_fbm(p))


@pytest.fixture(scope="module")
def fractal(orc):
    wl = workloads.config3(size=160, width=160, height=120, nviews=4)
    # closer cameras than the benchmark's so the sparse structures fill the small frames
    wl.views = workloads.orbit_views(4, 160, 120, radius=1.5 * workloads.DIAG, start=20.0)
    vol = orc.synth_fbm(wl.synth)
    assert np.array_equal(fbm_volume(wl.synth), vol)
    return wl, vol


def test_sparse_bricks_and_histograms(orc, fractal):
    wl, vol = fractal
    with Renderer() as r:
        r.loadVolume(vol, brick_size=24, overlap=2)   # 20^3 interiors: 8^3 bricks at 160^3
        mm = r.brickMinMax(0)
        empty = float((mm[:, 1] == 0).mean())
        assert 0.55 < empty < 0.85
        h1, f = orc.hist1d(vol)
        assert np.array_equal(r.getHistogram(), h1)
        h2, mg = orc.hist2d(vol, float(vol.max()), h1.size, f)
        g2, gmg = r.get2DHistogram()
        assert np.array_equal(g2, h2) and np.float32(mg) == np.float32(gmg)


def test_2d_tf_phong_matches_oracle(orc, fractal):
    wl, vol = fractal
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(wl.synth, brick_size=64, overlap=2)
        gmax = r.datasetInfo()["hist2d_max_grad"] * 0.5
        r.resize((wl.width, wl.height))
        r.setRenderMode(GBVR_RM_2DTRANS)
        r.set2DTrans(wl.tf, gmax)
        r.setValueRange(*wl.value_range)
        r.paintBatch(wl.views)
        imgs = [r.readFramebuffer(i, as_float=True) for i in range(len(wl.views))]
    for img, (v, p) in zip(imgs, wl.views):
        ref, _ = orc.render(vol, v, p, wl.width, wl.height, wl.tf, mode=1, grad_max=gmax,
                            value_range=wl.value_range)
        assert_close(img, ref)
    assert max(float(i[..., 3].max()) for i in imgs) > 0.2


def test_isosurfaces_match_oracle(orc, fractal):
    wl, vol = fractal
    v, p = wl.views[1]
    with Renderer(float_fb=True) as r:
        r.loadSynthetic(wl.synth, brick_size=64, overlap=2)
        r.resize((wl.width, wl.height))
        r.setRenderMode(GBVR_RM_ISOSURFACE)
        for iso in wl.isovalues:
            r.setIsoValue(iso, (0.8, 0.8, 0.9))
            r.setView(v, p)
            r.paint()
            img = r.readFramebuffer(0, as_float=True)
            ref, _ = orc.render(vol, v, p, wl.width, wl.height, np.zeros((2, 4), np.float32), mode=2, iso=iso,
                                iso_rgb=(0.8, 0.8, 0.9))
            hit_g, hit_r = img[..., 3] > 0.5, ref[..., 3] > 0.5
            assert (hit_g != hit_r).mean() < 0.002
            both = hit_g & hit_r
            assert_close(img[both], ref[both])
            assert hit_r.mean() > 0.003
