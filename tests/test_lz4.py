"""LZ4 block codec of the out-of-core brick store (host side): the library's
compressor round-trips through the library's decoder and through the
oracle's independent decoder; a block built by hand from the published format
decodes to its known text; malformed blocks are rejected."""
import ctypes as C

import numpy as np
import pytest

from imagevis3d_gb300 import _lib as L
from oracle import orc


def compress(data):
    lib = L.lib()
    src = np.frombuffer(data, np.uint8) if data else np.zeros(1, np.uint8)
    cap = lib.gbvr_lz4_bound(len(data))
    dst = np.zeros(cap, np.uint8)
    n = lib.gbvr_lz4_compress(src.ctypes.data, len(data), dst.ctypes.data, cap)
    assert n > 0
    return dst[:n].tobytes()


def decompress(block, out_n):
    src = np.frombuffer(block, np.uint8) if block else np.zeros(1, np.uint8)
    out = np.zeros(max(out_n, 1), np.uint8)
    rc = L.lib().gbvr_lz4_decompress(src.ctypes.data, len(block), out.ctypes.data, out_n)
    return out[:out_n].tobytes() if rc == 0 else None


def _cases():
    rng = np.random.default_rng(5)
    x = np.arange(65536)
    yield "empty", b""
    for n in (1, 5, 12, 13, 17, 20):
        yield "short%d" % n, bytes(rng.integers(0, 4, n, dtype=np.uint8))
    yield "zeros", bytes(65536)
    yield "random", rng.integers(0, 256, 65536, dtype=np.uint8).tobytes()
    yield "ramp16", (x // 97).astype(np.uint16).tobytes()[:65536]
    yield "smooth_u8", np.clip(128 + 60 * np.sin(x / 700.0) + rng.normal(0, 0.4, x.size), 0, 255).astype(np.uint8).tobytes()
    for period in (1, 2, 3, 7, 31, 32, 33, 300):
        yield "period%d" % period, (rng.integers(0, 256, period, dtype=np.uint8).tobytes() * (70000 // period))[:65536]
    yield "long_literals", rng.integers(0, 256, 300, dtype=np.uint8).tobytes() + bytes(2000)


@pytest.mark.parametrize("name,data", list(_cases()))
def test_round_trip_both_decoders(name, data):
    block = compress(data)
    assert decompress(block, len(data)) == data
    assert orc.lz4_decompress(block, len(data)) == data
    if name in ("zeros", "ramp16") or name.startswith("period"):
        assert len(block) < len(data) // 10


def test_hand_built_block():
    # token 0x35: 3 literals "abc", match of 5 + 4 = 9 bytes at offset 3 (it
    # overlaps its own output); token 0x20: 2 literals "de", the last sequence
    block = bytes([0x35]) + b"abc" + bytes([3, 0]) + bytes([0x20]) + b"de"
    assert decompress(block, 14) == b"abcabcabcabcde"
    assert orc.lz4_decompress(block, 14) == b"abcabcabcabcde"
    # 15 + 255 + 10 = 280 literals: the length continues over two bytes
    lit = bytes(range(256)) + bytes(24)
    block = bytes([0xF0, 255, 10]) + lit
    assert decompress(block, 280) == lit
    assert orc.lz4_decompress(block, 280) == lit


@pytest.mark.parametrize("block,n", [
    (b"", 4),                                        # no token
    (bytes([0x35]) + b"abc" + bytes([3]), 14),       # offset cut short
    (bytes([0x35]) + b"abc" + bytes([4, 0]) + bytes([0x20]) + b"de", 14),  # offset before the output
    (bytes([0x35]) + b"abc" + bytes([0, 0]) + bytes([0x20]) + b"de", 14),  # offset 0
    (bytes([0x50]) + b"abc", 5),                     # literals past the end
    (bytes([0x35]) + b"abc" + bytes([3, 0]), 12),    # ends with a match
    (bytes([0x35]) + b"abc" + bytes([3, 0]) + bytes([0x20]) + b"de", 13),  # too long for the output
])
def test_malformed_blocks_are_rejected(block, n):
    assert decompress(block, n) is None
    assert orc.lz4_decompress(block, n) is None or len(orc.lz4_decompress(block, n)) != n


def test_crafted_blocks_decode_on_the_host_as_the_reference():
    """The hand-built blocks of the GPU decoder's tests are valid LZ4: the
    library's host decoder and the plain Python reference agree on them."""
    from tests.lz4_blocks import cases, reference
    lib = L.lib()
    for i, blk in enumerate(cases()):
        ref = reference(blk)
        src = np.frombuffer(blk, np.uint8)
        out = np.zeros(len(ref), np.uint8)
        assert lib.gbvr_lz4_decompress(src.ctypes.data, len(blk), out.ctypes.data, len(ref)) == 0, i
        assert out.tobytes() == ref, i
