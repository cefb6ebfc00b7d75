"""UVF container I/O through the C ABI, host only (no GPU calls).

The writer must reproduce DemoData/c60.uvf byte for byte from its decoded
fields (layout: doc/import.adoc:904-1147 plus the raster tail of c60), and the
reader must recover every block and verify the MD5 over bytes 49..end
(ImageVis3D/UI/ImageVis3D_FileHandling.cpp:567-585).
"""
import ctypes as C
import hashlib
import os

import numpy as np
import pytest

from imagevis3d_gb300 import _lib as L
from tests.conftest import reference_file

RASTER_ID = b"Qvis data volume converted from C60Large.dat by ImageVis3D"


def write_c60(c60, path):
    vol = np.ascontiguousarray(c60["volume"])
    dims = (C.c_int64 * 3)(128, 128, 128)
    h1 = np.ascontiguousarray(c60["hist1d"], np.uint64)
    h2 = np.ascontiguousarray(c60["hist2d"], np.uint64)
    mm = np.ascontiguousarray(c60["minmax"], np.float64)
    L.call("gbvr_uvf_write_raster", path.encode(), RASTER_ID, vol.ctypes.data_as(C.c_void_p), dims,
           L.GBVR_U8, 256, 2, h1.ctypes.data_as(L.U64P), h1.size, h2.ctypes.data_as(L.U64P), 256, 256,
           float(c60["maxgrad_f32"][0]), mm.ctypes.data_as(C.POINTER(C.c_double)), 1)


def test_writer_reproduces_c60_bytes(c60, tmp_path):
    p = str(tmp_path / "c60_rewritten.uvf")
    write_c60(c60, p)
    data = open(p, "rb").read()
    assert len(data) == int(c60["file_size"][0])
    assert hashlib.md5(data).digest() == bytes(c60["file_md5"])
    assert data[33:49] == bytes(c60["checksum"])


def test_reader_roundtrip_and_verify(c60, tmp_path):
    p = str(tmp_path / "c60.uvf")
    write_c60(c60, p)
    s = L.UvfSummary()
    L.call("gbvr_uvf_inspect", p.encode(), 1, C.byref(s))
    assert s.version == 2 and s.checksum_semantic == 2 and s.checksum_verified == 1
    assert list(s.block_semantics[:s.nblocks]) == [1, 5, 6, 7]
    assert tuple(s.dims) == (128, 128, 128) and s.dtype == L.GBVR_U8 and s.lod_count == 1
    assert tuple(s.overlap) == (4, 4, 4) and s.data_offset == 484
    assert s.hist1d_size == 256 and (s.hist2d_nx, s.hist2d_ny) == (256, 256)
    assert np.float32(s.hist2d_max_grad) == c60["maxgrad_f32"][0]
    vol = np.empty((128, 128, 128), np.uint8)
    L.call("gbvr_uvf_read_volume", p.encode(), vol.ctypes.data_as(C.c_void_p), vol.nbytes)
    assert np.array_equal(vol, c60["volume"])
    h1 = np.zeros(256, np.uint64)
    L.call("gbvr_uvf_read_hist1d", p.encode(), h1.ctypes.data_as(L.U64P), 256)
    assert np.array_equal(h1, c60["hist1d"])
    h2 = np.zeros(65536, np.uint64)
    mg = C.c_float()
    L.call("gbvr_uvf_read_hist2d", p.encode(), h2.ctypes.data_as(L.U64P), h2.size, C.byref(mg))
    assert np.array_equal(h2.reshape(256, 256), c60["hist2d"])


def test_reader_on_reference_file(c60):
    path = reference_file("DemoData/c60.uvf")
    s = L.UvfSummary()
    L.call("gbvr_uvf_inspect", path.encode(), 1, C.byref(s))
    assert s.checksum_verified == 1
    assert bytes(s.checksum) == bytes(c60["checksum"])


def test_corrupt_checksum_is_reported(c60, tmp_path):
    p = str(tmp_path / "bad.uvf")
    write_c60(c60, p)
    raw = bytearray(open(p, "rb").read())
    raw[1000] ^= 0xFF  # one voxel
    open(p, "wb").write(bytes(raw))
    s = L.UvfSummary()
    with pytest.raises(L.GbvrError) as e:
        L.call("gbvr_uvf_inspect", p.encode(), 1, C.byref(s))
    assert e.value.code == -6
    # quick open (no verify) still parses
    L.call("gbvr_uvf_inspect", p.encode(), 0, C.byref(s))


def test_truncated_and_foreign_files(c60, tmp_path):
    p = str(tmp_path / "trunc.uvf")
    write_c60(c60, p)
    raw = open(p, "rb").read()
    open(p, "wb").write(raw[:5000])
    s = L.UvfSummary()
    with pytest.raises(L.GbvrError) as e:
        L.call("gbvr_uvf_inspect", p.encode(), 0, C.byref(s))
    assert e.value.code == -5
    q = str(tmp_path / "foreign.uvf")
    open(q, "wb").write(b"NOT-A-UVF" + bytes(100))
    with pytest.raises(L.GbvrError) as e:
        L.call("gbvr_uvf_inspect", q.encode(), 0, C.byref(s))
    assert e.value.code == -5
    with pytest.raises(L.GbvrError) as e:
        L.call("gbvr_uvf_inspect", str(tmp_path / "missing.uvf").encode(), 0, C.byref(s))
    assert e.value.code == -4
