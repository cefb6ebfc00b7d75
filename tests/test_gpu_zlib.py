"""The GPU zlib decoder (one warp per stream) on streams written by Python's
zlib module -- an independent encoder -- at every level (stored, fixed and
dynamic Huffman blocks) and on the library's own streams, in one batch;
every output equals the input bit for bit.  A corrupted stream, a wrong
checksum or a wrong output length raise the error flag, and the other
streams of the batch still decode."""
import ctypes as C
import zlib

import numpy as np
import pytest

from imagevis3d_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _inputs():
    rng = np.random.default_rng(17)
    x = np.arange(16384)
    out = [b"", b"a", b"abcabcabcabcabc" * 3, bytes(16384), rng.integers(0, 256, 16384, dtype=np.uint8).tobytes(),
           (x // 61).astype(np.uint16).tobytes()[:16384],
           np.clip(128 + 60 * np.sin(x / 300.0) + rng.normal(0, 1.5, x.size), 0, 255).astype(np.uint8).tobytes(),
           bytes((i * 13) % 251 for i in range(12000)), b"zlib brick " * 1400]
    return out


def _library_compress(data):
    lib = L.lib()
    src = np.frombuffer(data, np.uint8) if data else np.zeros(1, np.uint8)
    cap = lib.gbvr_zlib_bound(len(data))
    dst = np.zeros(cap, np.uint8)
    n = lib.gbvr_zlib_compress(src.ctypes.data, len(data), dst.ctypes.data, cap)
    assert n > 0
    return dst[:n].tobytes()


def _decode(torch, streams, raws, stored=None):
    """Decode streams on the GPU in one call; returns (outputs, error flag)."""
    stored = stored or [False] * len(streams)
    src = b"".join(streams)
    chunks = np.zeros((len(streams), 3), np.uint64)  # src, dst, comp | raw << 32
    so = do = 0
    for i, (s, r, st) in enumerate(zip(streams, raws, stored)):
        comp = len(s) | (0x80000000 if st else 0)
        chunks[i] = (so, do, comp | (r << 32))
        so += len(s)
        do += r
    d_src = torch.tensor(np.frombuffer(src + b"\0", np.uint8).copy(), device="cuda")
    d_dst = torch.zeros(max(do, 1), dtype=torch.uint8, device="cuda")
    d_chunks = torch.tensor(chunks.view(np.int64), device="cuda")
    d_err = torch.zeros(1, dtype=torch.int32, device="cuda")
    L.call("gbvr_dev_zlib_decode", C.c_void_p(d_src.data_ptr()), C.c_void_p(d_dst.data_ptr()),
           C.c_void_p(d_chunks.data_ptr()), len(streams), C.c_void_p(d_err.data_ptr()), None)
    torch.cuda.synchronize()
    out = d_dst.cpu().numpy().tobytes()
    res, o = [], 0
    for r in raws:
        res.append(out[o:o + r])
        o += r
    return res, int(d_err.item())


def _all_streams():
    datas = _inputs()
    streams, raws, labels = [], [], []
    for j, d in enumerate(datas):
        for level in (0, 1, 6, 9):
            streams.append(zlib.compress(d, level))
            raws.append(len(d))
            labels.append("input %d, zlib level %d" % (j, level))
        streams.append(_library_compress(d))
        raws.append(len(d))
        labels.append("input %d, library" % j)
    return datas, streams, raws, labels


def test_gpu_decodes_each_stream():
    torch = pytest.importorskip("torch")
    datas, streams, raws, labels = _all_streams()
    for k, (st, r, lab) in enumerate(zip(streams, raws, labels)):
        out, err = _decode(torch, [st], [r])
        assert err == 0, lab
        assert out[0] == datas[k // 5], lab


def test_gpu_decodes_zlib_and_library_streams_in_one_batch():
    torch = pytest.importorskip("torch")
    datas, streams, raws, labels = _all_streams()
    # and one chunk stored raw
    streams.append(datas[4])
    raws.append(len(datas[4]))
    stored = [False] * (len(streams) - 1) + [True]
    out, err = _decode(torch, streams, raws, stored)
    assert err == 0
    for k in range(len(streams) - 1):
        assert out[k] == datas[k // 5], labels[k]
    assert out[-1] == datas[4]


@pytest.mark.parametrize("damage", ["checksum", "truncated", "length", "bits"])
def test_gpu_decoder_flags_malformed_streams(damage):
    torch = pytest.importorskip("torch")
    data = bytes(range(256)) * 40
    good = zlib.compress(data, 6)
    bad = bytearray(good)
    raw = len(data)
    if damage == "checksum":
        bad[-1] ^= 1
    elif damage == "truncated":
        bad = bad[:len(bad) // 2]
    elif damage == "length":
        raw = len(data) - 1
    else:
        bad[len(bad) // 3] ^= 0x5A
    out, err = _decode(torch, [good, bytes(bad), good], [len(data), raw, len(data)])
    assert err != 0
    assert out[0] == data and out[2] == data  # the other streams of the batch decode
