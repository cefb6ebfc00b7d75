"""zlib / DEFLATE codec of the out-of-core brick store (host side), checked
against Python's zlib module, an independent implementation of the same
formats (RFC 1950 / 1951): the library's streams decompress with zlib, zlib's
streams at every level (stored, fixed and dynamic Huffman blocks)
decompress with the library, and malformed streams are rejected."""
import zlib

import numpy as np
import pytest

from imagevis3d_gb300 import _lib as L

EFORMAT = -5


def compress(data):
    lib = L.lib()
    src = np.frombuffer(data, np.uint8) if data else np.zeros(1, np.uint8)
    cap = lib.gbvr_zlib_bound(len(data))
    dst = np.zeros(cap, np.uint8)
    n = lib.gbvr_zlib_compress(src.ctypes.data, len(data), dst.ctypes.data, cap)
    assert n > 0
    return dst[:n].tobytes()


def decompress(stream, out_n):
    src = np.frombuffer(stream, np.uint8) if stream else np.zeros(1, np.uint8)
    out = np.zeros(max(out_n, 1), np.uint8)
    rc = L.lib().gbvr_zlib_decompress(src.ctypes.data, len(stream), out.ctypes.data, out_n)
    return out[:out_n].tobytes() if rc == 0 else rc


def cases():
    rng = np.random.default_rng(11)
    x = np.arange(70000)
    yield "empty", b""
    for n in (1, 2, 3, 7, 40):
        yield "short%d" % n, bytes(rng.integers(0, 3, n, dtype=np.uint8))
    yield "zeros", bytes(100000)
    yield "random", rng.integers(0, 256, 70000, dtype=np.uint8).tobytes()
    yield "ramp16", (x // 97).astype(np.uint16).tobytes()
    yield "smooth_u8", np.clip(128 + 60 * np.sin(x / 700.0) + rng.normal(0, 2.0, x.size), 0, 255).astype(
        np.uint8).tobytes()
    yield "periodic", bytes((i * 7) % 251 for i in range(20000))
    yield "text", b"ImageVis3D brick " * 3000


CASES = list(cases())
IDS = [name for name, _ in CASES]


@pytest.mark.parametrize("name,data", CASES, ids=IDS)
def test_library_streams_decompress_with_zlib(name, data):
    c = compress(data)
    assert zlib.decompress(c) == data
    assert decompress(c, len(data)) == data
    if name in ("zeros", "ramp16", "periodic", "text"):
        # within 25% of zlib's own default level
        assert len(c) <= 1.25 * len(zlib.compress(data, 6)) + 16, (name, len(c))
    if name == "random":
        assert len(c) <= L.lib().gbvr_zlib_bound(len(data))  # stored blocks, at most the stated bound


@pytest.mark.parametrize("level", [0, 1, 6, 9])
@pytest.mark.parametrize("name,data", CASES, ids=IDS)
def test_zlib_streams_decompress_with_the_library(name, data, level):
    c = zlib.compress(data, level)
    assert decompress(c, len(data)) == data


def test_fixed_huffman_block():
    # a short input zlib codes with the fixed Huffman codes (block type 1)
    data = b"abcabcabcabcabc" * 3
    c = zlib.compress(data, 9)
    assert (c[2] >> 1) & 3 == 1  # BTYPE of the first block
    assert decompress(c, len(data)) == data


def test_malformed_streams_are_rejected():
    data = bytes(range(256)) * 40
    c = bytearray(zlib.compress(data, 6))
    assert decompress(bytes(c[:-1]), len(data)) == EFORMAT       # truncated checksum
    assert decompress(bytes(c[:len(c) // 2]), len(data)) == EFORMAT  # truncated data
    bad = bytearray(c)
    bad[-1] ^= 1                                                 # wrong Adler-32
    assert decompress(bytes(bad), len(data)) == EFORMAT
    bad = bytearray(c)
    bad[0] = 0x79                                                # header check fails
    assert decompress(bytes(bad), len(data)) == EFORMAT
    assert decompress(bytes(c), len(data) - 1) == EFORMAT       # longer than the output
    assert decompress(bytes(c), len(data) + 1) == EFORMAT       # shorter than the output
    stored = zlib.compress(data, 0)
    bad = bytearray(stored)
    bad[5] ^= 0xFF                                               # LEN / NLEN disagree
    assert decompress(bytes(bad), len(data)) == EFORMAT
    rng = np.random.default_rng(3)
    for _ in range(200):                                         # random corruption never crashes
        bad = bytearray(c)
        for p in rng.integers(2, len(c), 3):
            bad[p] = int(rng.integers(0, 256))
        r = decompress(bytes(bad), len(data))
        assert r == EFORMAT or r == data
