"""GPU UVF build (bricking with ghosts, LOD pyramid, per-brick min/max, 1D and
2D histograms, seeded synthesis) against the CPU oracle, bit for bit, and
against the reference's c60.uvf."""
import hashlib
import os

import numpy as np
import pytest

from imagevis3d_gb300 import Renderer, synth_params, synth_volume, workloads
from tests.test_uvf_host import write_c60

pytestmark = pytest.mark.gpu


def test_synth_u8_matches_oracle(orc):
    sp = workloads.config1().synth
    assert np.array_equal(synth_volume(sp), orc.synth_blobs(sp))


def test_synth_u16_background_gaussian_noise_matches_oracle(orc):
    sp = synth_params((96, 80, 72), np.uint16, 77, 16, (5.0, 20.0), (0.3, 1.0), 2600.0,
                      noise_kind=2, noise_amp=20.0, vmax=4095.0, bg_freq=1.0, bg_level=0.15,
                      bg_amp=0.1)
    g = synth_volume(sp)
    assert np.array_equal(g, orc.synth_blobs(sp))
    assert g.max() > 1000


def test_c60_build_bit_exact(c60):
    with Renderer() as r:
        r.loadVolume(c60["volume"], brick_size=256, overlap=2)
        info = r.datasetInfo()
        assert info["lod_count"] == 1 and info["lod_bricks"][0] == (1, 1, 1)
        assert np.array_equal(r.getHistogram(), c60["hist1d"])
        h2, mg = r.get2DHistogram()
        assert np.array_equal(h2, c60["hist2d"])
        assert np.float32(mg) == c60["maxgrad_f32"][0]
        mm = r.brickMinMax(0)
        assert tuple(mm[0]) == (c60["minmax"][0], c60["minmax"][1])
        b, o = r.getBrick(0, (0, 0, 0))
        # one brick: the level plus 2 replicated ghost voxels per face
        assert o == (-2, -2, -2) and np.array_equal(b[2:-2, 2:-2, 2:-2], c60["volume"])
        assert np.array_equal(b, np.pad(c60["volume"], 2, mode="edge"))


def test_c60_load_uvf_and_write_back_byte_exact(c60, tmp_path):
    src = str(tmp_path / "c60.uvf")
    write_c60(c60, src)
    out = str(tmp_path / "c60_gpu.uvf")
    with Renderer() as r:
        r.loadDataset(src)
        r.writeUVF(out)
    data = open(out, "rb").read()
    assert hashlib.md5(data).digest() == bytes(c60["file_md5"])


def _levels(orc, vol, brick, ghost):
    dims = (vol.shape[2], vol.shape[1], vol.shape[0])
    lv = [vol]
    for d in orc.lod_dims(dims, brick, ghost)[1:]:
        lv.append(orc.downsample(lv[-1]))
        assert (lv[-1].shape[2], lv[-1].shape[1], lv[-1].shape[0]) == d
    return lv


@pytest.mark.parametrize("dtype,shape,brick", [(np.uint16, (110, 130, 150), 64),
                                               (np.uint8, (70, 64, 97), 32)])
def test_multibrick_pyramid_bit_exact(orc, dtype, shape, brick):
    sp = synth_params((shape[2], shape[1], shape[0]), dtype, 5, 12, (4.0, 16.0), (0.3, 1.0),
                      2600.0 if dtype == np.uint16 else 255.0, noise_kind=1, noise_amp=6.0,
                      vmax=4095.0 if dtype == np.uint16 else 255.0)
    vol = orc.synth_blobs(sp)
    lv = _levels(orc, vol, brick, 2)
    with Renderer() as r:
        r.loadVolume(vol, brick_size=brick, overlap=2)
        info = r.datasetInfo()
        assert info["lod_count"] == len(lv)
        for l, level in enumerate(lv):
            nb, _ = orc.brick_grid((level.shape[2], level.shape[1], level.shape[0]), brick, 2)
            assert info["lod_bricks"][l] == nb
            mm = r.brickMinMax(l)
            i = 0
            for bz in range(nb[2]):
                for by in range(nb[1]):
                    for bx in range(nb[0]):
                        want, wo = orc.extract_brick(level, brick, 2, (bx, by, bz))
                        got, go = r.getBrick(l, (bx, by, bz))
                        assert go == wo and np.array_equal(got, want), (l, bx, by, bz)
                        assert mm[i, 0] == want.min() and mm[i, 1] == want.max()
                        i += 1
        h1, f = orc.hist1d(vol)
        assert np.array_equal(r.getHistogram(), h1)
        h2, mg = orc.hist2d(vol, float(vol.max()), h1.size, f)
        g2, gmg = r.get2DHistogram()
        assert np.array_equal(g2, h2) and np.float32(mg) == np.float32(gmg)


def test_hist_merge_for_wide_16bit_range(orc):
    rng = np.random.default_rng(3)
    vol = rng.integers(0, 10001, (40, 50, 60), dtype=np.uint16)
    vol[0, 0, 0] = 10000
    h1, f = orc.hist1d(vol)
    assert f == 3
    with Renderer() as r:
        r.loadVolume(vol, brick_size=64, overlap=2)
        assert np.array_equal(r.getHistogram(), h1)
        h2, mg = orc.hist2d(vol, 10000.0, h1.size, f)
        g2, gmg = r.get2DHistogram()
        assert np.array_equal(g2, h2) and np.float32(mg) == np.float32(gmg)


def test_constant_and_tiny_volumes(orc):
    for vol in (np.full((9, 10, 11), 7, np.uint8), np.zeros((1, 1, 1), np.uint16),
                np.arange(8, dtype=np.uint8).reshape(2, 2, 2)):
        with Renderer() as r:
            r.loadVolume(vol, brick_size=32, overlap=2)
            h1, f = orc.hist1d(vol)
            assert np.array_equal(r.getHistogram(), h1)
            h2, mg = orc.hist2d(vol, float(vol.max()), h1.size, f)
            g2, gmg = r.get2DHistogram()
            assert np.array_equal(g2, h2) and np.float32(gmg) == np.float32(mg)
