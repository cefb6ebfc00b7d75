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


@pytest.mark.parametrize("top", [16383, 16384])
def test_hist2d_of_16bit_volumes_at_the_32bit_sum_limit(orc, top):
    """A build's 2D histogram sums squared differences in 32 bits when the
    16-bit volume's largest value is below 16384, and in 64 bits otherwise:
    both equal the rule bit for bit at the extreme gradients next to that
    limit (voxels alternating between 0 and the top value)."""
    rng = np.random.default_rng(top)
    vol = np.where(rng.random((40, 36, 64)) < 0.5, 0, top).astype(np.uint16)
    vol[5:9, 4:30, 10:50] = rng.integers(0, top + 1, (4, 26, 40), dtype=np.uint16)
    vol[0, 0, 0] = top
    with Renderer() as r:
        r.loadVolume(vol, brick_size=32, overlap=2)
        h1, f = orc.hist1d(vol)
        assert np.array_equal(r.getHistogram(), h1)
        h2, mg = orc.hist2d(vol, float(top), h1.size, f)
        g2, gmg = r.get2DHistogram()
        assert np.array_equal(g2, h2) and np.float32(gmg) == np.float32(mg)


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


def _dev_hist2d(vol, max_scalar, nx, merge, offset=0):
    import ctypes as C
    import torch
    from imagevis3d_gb300 import _lib as L
    flat = torch.from_numpy(np.ascontiguousarray(vol).reshape(-1).view(np.uint8))
    buf = torch.zeros(flat.numel() + 16, dtype=torch.uint8, device="cuda")
    buf[offset:offset + flat.numel()] = flat.cuda()
    hist = torch.zeros(nx * 256, dtype=torch.int64, device="cuda")
    dims = (C.c_int64 * 3)(vol.shape[2], vol.shape[1], vol.shape[0])
    mg = C.c_float()
    L.call("gbvr_dev_hist2d", C.c_void_p(buf.data_ptr() + offset), 0 if vol.dtype == np.uint8 else 1, dims,
           max_scalar, nx, merge, C.c_void_p(hist.data_ptr()), C.byref(mg), None)
    torch.cuda.synchronize()
    return hist.cpu().numpy().astype(np.uint64).reshape(nx, 256), mg.value


def _hist2d_cases(orc):
    blobs = lambda dims, dt, vmax, scale: orc.synth_blobs(
        synth_params(dims, dt, 9, 10, (3.0, 9.0), (0.3, 1.0), scale, noise_kind=1, noise_amp=3.0, vmax=vmax))
    z, y, x = np.meshgrid(np.arange(20), np.arange(30), np.arange(40), indexing="ij")
    return {
        "u8_smem": (blobs((200, 64, 48), np.uint8, 255.0, 255.0), 0),
        "u8_periodic_flush": (blobs((16384, 64, 16), np.uint8, 255.0, 255.0), 0),
        "u8_x4": (blobs((4, 30, 20), np.uint8, 255.0, 255.0), 0),
        "u8_misaligned": (blobs((200, 64, 48), np.uint8, 255.0, 255.0), 1),
        "u8_ramp_ties": (((x + y + z) % 200).astype(np.uint8), 0),
        "u16_smem": (blobs((96, 50, 40), np.uint16, 200.0, 200.0), 0),
        "u16_global": (blobs((128, 40, 36), np.uint16, 4095.0, 2600.0), 0),
        "u8_deep": (blobs((64, 8, 300), np.uint8, 255.0, 255.0), 0),
        "u16_wide_nosmem": (blobs((64, 20, 10), np.uint16, 16000.0, 16000.0), 0),
        # z split into segments (4 of 33 planes, the last 31; 3 of 34, the
        # last 32; 2 of 35): columns restart mid-volume
        "u16_zsegments": (blobs((96, 40, 130), np.uint16, 4095.0, 2600.0), 0),
        "u8_ramp_ties_zsegments": ((np.add.outer(np.arange(100), np.add.outer(np.arange(30), np.arange(40))) % 200)
                                   .astype(np.uint8), 0),
        "u16_wide_nosmem_zsegments": (blobs((64, 12, 70), np.uint16, 16000.0, 16000.0), 0),
    }


@pytest.mark.parametrize("case", ["u8_smem", "u8_periodic_flush", "u8_x4", "u8_misaligned", "u8_ramp_ties",
                                  "u16_smem", "u16_global", "u8_deep", "u16_wide_nosmem", "u16_zsegments",
                                  "u8_ramp_ties_zsegments", "u16_wide_nosmem_zsegments"])
def test_dev_hist2d_paths_bit_exact(orc, case):
    vol, offset = _hist2d_cases(orc)[case]
    h1, f = orc.hist1d(vol)
    nx = h1.size
    if case.startswith("u16_wide_nosmem"):
        nx, f = int(vol.max()) + 1, 1  # 16001 value bins: no gradient row fits in shared memory
    ms = float(vol.max())
    want, wmg = orc.hist2d(vol, ms, nx, f)
    got, gmg = _dev_hist2d(vol, ms, nx, f, offset)
    assert np.array_equal(got, want), case
    assert np.float32(gmg) == np.float32(wmg)


def _cell_ranges(vol, m):
    """Macro-cell (min, max) of a (z, y, x) level: cell c covers voxels
    [c m - 1, c m + m + 1] per axis, clamped to the level (edge padding
    repeats the edge voxel, which the clamped range already holds)."""
    lo, hi = vol.astype(np.float32), vol.astype(np.float32)
    for ax in range(3):
        n = vol.shape[ax]
        nc = -(-n // m)
        pad = [(0, 0)] * 3
        pad[ax] = (1, nc * m + 2 - n)
        win = [np.lib.stride_tricks.sliding_window_view(np.pad(a, pad, mode="edge"), m + 3, axis=ax)
               for a in (lo, hi)]
        sl = [slice(None)] * 3
        sl[ax] = slice(0, nc * m, m)
        lo, hi = win[0][tuple(sl)].min(axis=-1), win[1][tuple(sl)].max(axis=-1)
    return np.stack([lo, hi], axis=-1)


@pytest.mark.parametrize("dtype,shape,brick,layouts", [(np.uint16, (37, 50, 23), 32, 4),
                                                       (np.uint8, (70, 64, 97), 32, 6),
                                                       (np.float32, (29, 41, 66), 64, 1),
                                                       # 16-bit rows of whole 4-byte words: the tiles
                                                       # away from the x faces read their rows as words
                                                       (np.uint16, (21, 30, 128), 64, 4),
                                                       (np.uint8, (19, 27, 136), 64, 1)])
def test_macro_cell_ranges_and_brick_minmax_bit_exact(orc, dtype, shape, brick, layouts):
    """The macro-cell min/max grid of every level (the skipping structure) and
    each brick's min/max over its stored voxels equal their rules bit for bit,
    for sizes that are not multiples of the cell edge, every layout copy
    choice, and float data with negative values."""
    rng = np.random.default_rng(11)
    if dtype == np.float32:
        vol = (rng.normal(0.0, 40.0, shape) - 15.0).astype(np.float32)
    else:
        top = 4095 if dtype == np.uint16 else 255
        vol = rng.integers(0, top + 1, shape).astype(dtype)
    lv = _levels(orc, vol, brick, 2)
    with Renderer() as r:
        r.loadVolume(vol, brick_size=brick, overlap=2, layouts=layouts)
        for l, level in enumerate(lv):
            got, edge = r.cellMinMax(l)
            assert edge == 4
            assert np.array_equal(got, _cell_ranges(level, 4)), l
            nb, _ = orc.brick_grid((level.shape[2], level.shape[1], level.shape[0]), brick, 2)
            mm = r.brickMinMax(l)
            i = 0
            for bz in range(nb[2]):
                for by in range(nb[1]):
                    for bx in range(nb[0]):
                        want, _ = orc.extract_brick(level, brick, 2, (bx, by, bz))
                        assert mm[i, 0] == want.min() and mm[i, 1] == want.max(), (l, bx, by, bz)
                        i += 1
