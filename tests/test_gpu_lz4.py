"""The GPU LZ4 decoder (one warp per block, the decoder of paged bricks) on
blocks written by the library's compressor and on hand-built blocks whose
sequences reach every copy path: offsets 1 .. 31 (periodic copies), offsets
of 32 and more with short and long matches (single-step sequences and
32-byte steps), offsets above 480 and up to 4000, literal runs above 15 and
255 bytes, stored chunks, and outputs above 16 KiB.  Every output equals its
reference (a plain Python decoder of the block format) bit for bit; a block
that does not produce its chunk's length sets the error flag while the
others still decode."""
import ctypes as C

import numpy as np
import pytest

from imagevis3d_gb300 import _lib as L
from tests.lz4_blocks import cases, dense, reference

pytestmark = pytest.mark.gpu


def _decode(torch, blocks, raws, stored=None):
    stored = stored or [False] * len(blocks)
    src = b"".join(blocks)
    chunks = np.zeros((len(blocks), 3), np.uint64)  # src, dst, comp | raw << 32
    so = do = 0
    for i, (s, r, st) in enumerate(zip(blocks, raws, stored)):
        chunks[i] = (so, do, (len(s) | (0x80000000 if st else 0)) | (r << 32))
        so += len(s)
        do += r
    d_src = torch.tensor(np.frombuffer(src + b"\0", np.uint8).copy(), device="cuda")
    d_dst = torch.zeros(max(do, 1), dtype=torch.uint8, device="cuda")
    d_chunks = torch.tensor(chunks.view(np.int64), device="cuda")
    d_err = torch.zeros(1, dtype=torch.int32, device="cuda")
    L.call("gbvr_dev_lz4_decode", C.c_void_p(d_src.data_ptr()), C.c_void_p(d_dst.data_ptr()),
           C.c_void_p(d_chunks.data_ptr()), len(blocks), C.c_void_p(d_err.data_ptr()), None)
    torch.cuda.synchronize()
    out = d_dst.cpu().numpy().tobytes()
    res, o = [], 0
    for r in raws:
        res.append(out[o:o + r])
        o += r
    return res, int(d_err.item())


def test_gpu_decodes_every_copy_path():
    torch = pytest.importorskip("torch")
    blocks = cases()
    refs = [reference(b) for b in blocks]
    assert max(len(r) for r in refs) > 16384
    got, err = _decode(torch, blocks, [len(r) for r in refs])
    assert err == 0
    for i, (g, r) in enumerate(zip(got, refs)):
        assert g == r, i


def test_stored_chunks_and_a_malformed_block():
    torch = pytest.importorskip("torch")
    blocks = cases()[:3]
    refs = [reference(b) for b in blocks]
    raw = np.random.default_rng(5).integers(0, 256, 5000, dtype=np.uint8).tobytes()
    got, err = _decode(torch, blocks + [raw], [len(r) for r in refs] + [len(raw)], [False] * 3 + [True])
    assert err == 0 and got[3] == raw and all(g == r for g, r in zip(got, refs))
    # a block that does not produce exactly its chunk's length is malformed;
    # the other blocks of the batch still decode
    got, err = _decode(torch, blocks, [len(refs[0]), len(refs[1]) + 7, len(refs[2])])
    assert err != 0
    assert got[0] == refs[0] and got[2] == refs[2]


def test_malformed_sequence_inside_a_window_of_short_sequences():
    """An offset of 0 among short sequences (decoded several per 32 input
    bytes), and a chunk whose length ends inside such a window: both set the
    error flag; the good blocks of the batch still decode."""
    torch = pytest.importorskip("torch")
    good = dense(21)
    ref = reference(good)
    bad = dense(21, zero_offset_at=350)
    got, err = _decode(torch, [good, bad, good], [len(ref), len(ref), len(ref)])
    assert err != 0
    assert got[0] == ref and got[2] == ref
    got, err = _decode(torch, [good, good], [len(ref), len(ref) // 2])
    assert err != 0 and got[0] == ref
