"""The 1024^3 uint16 bricked workload at full size: size-independent
properties of the GPU build, and a seeded pixel subset of full-resolution
views against the FP64 oracle."""
import numpy as np
import pytest

from imagevis3d_gb300 import Renderer, synth_volume, workloads
from tests.gpu_util import assert_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c2():
    wl = workloads.config2()
    vol = synth_volume(wl.synth)
    r = Renderer(float_fb=True)
    r.loadSynthetic(wl.synth, **wl.brick)
    r.resize((wl.width, wl.height))
    r.set1DTrans(wl.tf)
    r.setValueRange(*wl.value_range)
    r.setSampleRateModifier(wl.spv)
    yield wl, vol, r
    r.cleanup()


def test_pyramid_and_histograms(c2):
    wl, vol, r = c2
    info = r.datasetInfo()
    assert info["lod_count"] == 4
    assert info["lod_dims"] == [(1024,) * 3, (512,) * 3, (256,) * 3, (128,) * 3]
    assert info["lod_bricks"] == [(5, 5, 5), (3, 3, 3), (2, 2, 2), (1, 1, 1)]
    h1 = r.getHistogram()
    assert int(h1.sum()) == 1024 ** 3 and h1.size == int(vol.max()) + 1
    assert np.array_equal(np.bincount(vol.ravel(), minlength=h1.size).astype(np.uint64), h1)
    h2, mg = r.get2DHistogram()
    assert np.array_equal(h2.sum(axis=1), h1) and mg > 0
    assert info["range"] == (float(vol.min()), float(vol.max()))


def test_full_size_2d_histogram_equals_the_rule(orc, c2):
    """The 2D histogram of the whole 1024^3 level (12-bit values: gradient
    sums in 32 bits) and its max gradient equal the FP64 restatement of the
    rule bit for bit (about 40 s of CPU)."""
    wl, vol, r = c2
    h1, f = orc.hist1d(vol)
    want, wmg = orc.hist2d(vol, float(vol.max()), h1.size, f)
    got, gmg = r.get2DHistogram()
    assert np.array_equal(got, want) and np.float32(gmg) == np.float32(wmg)


def test_bricks_tile_the_volume_with_exact_ghosts(c2):
    wl, vol, r = c2
    mm = r.brickMinMax(0)
    rng = np.random.default_rng(7)
    picks = [(0, 0, 0), (4, 4, 4)] + [tuple(int(x) for x in rng.integers(0, 5, 3)) for _ in range(4)]
    for b in picks:
        data, o = r.getBrick(0, b)
        # stored box = interior + 2 ghosts per face, edge voxels replicated
        zi = np.clip(np.arange(o[2], o[2] + data.shape[0]), 0, 1023)
        yi = np.clip(np.arange(o[1], o[1] + data.shape[1]), 0, 1023)
        xi = np.clip(np.arange(o[0], o[0] + data.shape[2]), 0, 1023)
        assert np.array_equal(data, vol[np.ix_(zi, yi, xi)])
        i = (b[2] * 5 + b[1]) * 5 + b[0]
        assert mm[i, 0] == data.min() and mm[i, 1] == data.max()


def test_full_resolution_views_match_oracle_on_pixel_subset(orc, c2):
    wl, vol, r = c2
    views = wl.views[::16]  # 4 of the 64 orbit views
    r.paintBatch(views)
    rng = np.random.default_rng(wl.synth.seed)
    for i, (v, p) in enumerate(views):
        img = r.readFramebuffer(i, as_float=True).reshape(-1, 4)
        alpha = img[:, 3]
        # half the subset on covered pixels, half anywhere
        cov = np.flatnonzero(alpha > 0.02)
        pix = np.concatenate([rng.choice(cov, 600, replace=False), rng.integers(0, img.shape[0], 200)])
        ref, _ = orc.render(vol, v, p, wl.width, wl.height, wl.tf, spv=wl.spv,
                            value_range=wl.value_range, pixels=pix)
        assert_close(img[pix], ref)
