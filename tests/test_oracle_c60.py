"""Pin the CPU oracle against the reference's own UVF output (DemoData/c60.uvf).

c60.uvf is a 128^3 uint8 volume written by ImageVis3D's converter with its
1D histogram, 2D histogram (value x gradient magnitude) and min/max block
(UVFReader/DataSource.h:601-657 is the sequence that produces those blocks).
"""
import numpy as np


def test_hist1d_matches_c60(c60, orc):
    h, f = orc.hist1d(c60["volume"])
    assert f == 1
    assert h.shape == c60["hist1d"].shape
    assert np.array_equal(h, c60["hist1d"])
    assert int(h.sum()) == 128 ** 3


def test_hist2d_matches_c60_bit_exact(c60, orc):
    vol = c60["volume"]
    h2, mg = orc.hist2d(vol, float(vol.max()), 256)
    assert np.array_equal(h2, c60["hist2d"])
    # the stored float32 max gradient
    assert np.float32(mg) == c60["maxgrad_f32"][0]
    # rows of the 2D histogram sum to the 1D histogram
    assert np.array_equal(h2.sum(axis=1), c60["hist1d"])


def test_minmax_matches_c60(c60, orc):
    mm = c60["minmax"]
    vol = c60["volume"]
    assert mm[0] == vol.min() and mm[1] == vol.max()
    assert mm[2] == -np.finfo(np.float64).max and mm[3] == np.finfo(np.float64).max


def test_c60_raster_header(c60):
    w = c60["raster_words"].astype(np.int64)
    assert list(w[20:23]) == [128, 128, 128]   # domain
    assert list(w[23:26]) == [256, 256, 256]   # brick size
    assert list(w[26:29]) == [4, 4, 4]         # overlap = 2 * DEFAULT_BRICKOVERLAP
    assert w[35] == 1                          # one LOD level


def test_lod_rule(orc):
    # 1024^3 with 256-voxel bricks incl. 2 ghosts: 1024, 512, 256, 128
    assert orc.lod_dims((1024, 1024, 1024), 256, 2) == [(1024,) * 3, (512,) * 3, (256,) * 3, (128,) * 3]
    # c60: fits one brick interior, one level
    assert orc.lod_dims((128, 128, 128), 256, 2) == [(128, 128, 128)]
    assert orc.lod_dims((300, 20, 7), 64, 2) == [(300, 20, 7), (150, 10, 4), (75, 5, 2), (38, 3, 1)]
    assert orc.lod_dims((1024,) * 3, 256, 2, max_lods=2) == [(1024,) * 3, (512,) * 3]


def test_brick_grid_and_ghosts(orc):
    rng = np.random.default_rng(1)
    vol = rng.integers(0, 4096, (70, 90, 130), dtype=np.uint16)  # z, y, x
    nb, interior = orc.brick_grid((130, 90, 70), 32, 2)
    assert interior == 28 and nb == (5, 4, 3)
    padded = np.pad(vol, 2, mode="edge")  # clamp-to-edge ghosts outside the level
    for b in [(0, 0, 0), (4, 3, 2), (2, 1, 1)]:
        data, o = orc.extract_brick(vol, 32, 2, b)
        for a, n in zip(range(3), (130, 90, 70)):
            lo = b[a] * 28
            hi = min(lo + 28, n)
            assert o[a] == lo - 2 and data.shape[2 - a] == hi - lo + 4
        z0, y0, x0 = o[2] + 2, o[1] + 2, o[0] + 2
        assert np.array_equal(data, padded[z0:z0 + data.shape[0], y0:y0 + data.shape[1], x0:x0 + data.shape[2]])
    # single-brick level: the whole level plus replicated ghosts
    small = vol[:20, :20, :20].copy()
    data, o = orc.extract_brick(small, 32, 2, (0, 0, 0))
    assert data.shape == (24, 24, 24) and o == (-2, -2, -2)
    assert np.array_equal(data, np.pad(small, 2, mode="edge"))


def test_downsample_rule(orc):
    v = np.array([[[1, 2, 3], [4, 5, 6]], [[7, 8, 9], [10, 11, 200]]], np.uint8)  # z=2, y=2, x=3
    d = orc.downsample(v)
    assert d.shape == (1, 1, 2)
    assert d[0, 0, 0] == (1 + 2 + 4 + 5 + 7 + 8 + 10 + 11) // 8
    assert d[0, 0, 1] == (3 + 6 + 9 + 200) // 4
    f = orc.downsample(v.astype(np.float32))
    assert f[0, 0, 1] == np.float32((3 + 6 + 9 + 200) / 4)


def test_hist1d_compress_rule(orc):
    v = np.arange(10000, dtype=np.uint16).reshape(10, 10, 100)
    h, f = orc.hist1d(v, max_bins=4096)
    assert f == 3 and h.size == 3334
    assert int(h.sum()) == 10000 and h[0] == 3 and h[-1] == 1


def test_hist2d_constant_volume(orc):
    v = np.full((5, 6, 7), 9, np.uint8)
    h2, mg = orc.hist2d(v, 9.0, 10)
    assert mg == 0.0 and h2[9, 0] == v.size and h2.sum() == v.size
