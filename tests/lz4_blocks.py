"""LZ4 blocks for the decoder tests: a writer of single sequences, a plain
decoder of the block format (the reference), blocks built from chosen
offsets and lengths so that every copy path of the GPU decoder is reached,
and blocks from the library's compressor."""
import numpy as np

from imagevis3d_gb300 import _lib as L


def lenext(r):
    out = bytearray()
    while r >= 255:
        out.append(255)
        r -= 255
    out.append(r)
    return bytes(out)


def sequence(lit, off, mlen):
    """One LZ4 sequence (mlen 0: the last one, literals only)."""
    ml = mlen - 4 if mlen else 0
    token = (min(len(lit), 15) << 4) | (min(ml, 15) if mlen else 0)
    out = bytes([token])
    if len(lit) >= 15:
        out += lenext(len(lit) - 15)
    out += lit
    if mlen:
        out += bytes([off & 255, off >> 8])
        if ml >= 15:
            out += lenext(ml - 15)
    return out


def reference(block):
    out = bytearray()
    ip = 0
    while True:
        t = block[ip]
        ip += 1
        nl = t >> 4
        if nl == 15:
            while True:
                b = block[ip]
                ip += 1
                nl += b
                if b != 255:
                    break
        out += block[ip:ip + nl]
        ip += nl
        if ip == len(block):
            return bytes(out)
        off = block[ip] | (block[ip + 1] << 8)
        ip += 2
        ml = t & 15
        if ml == 15:
            while True:
                b = block[ip]
                ip += 1
                ml += b
                if b != 255:
                    break
        for _ in range(ml + 4):
            out.append(out[-off])


def crafted(seed, offsets, lengths, n_seq, head=700, lits=(0, 1, 3, 14, 15, 16, 40, 300)):
    rng = np.random.default_rng(seed)
    block = b""
    out_len = 0
    lit = rng.integers(0, 256, head, dtype=np.uint8).tobytes()
    first = True
    for _ in range(n_seq):
        if not first:
            lit = rng.integers(0, 256, int(rng.choice(lits)), dtype=np.uint8).tobytes()
        first = False
        off = int(rng.choice(offsets))
        mlen = int(rng.choice(lengths))
        if off > out_len + len(lit):
            off = out_len + len(lit)
        block += sequence(lit, off, mlen)
        out_len += len(lit) + mlen
    block += sequence(b"tail!", 0, 0)
    return block


def dense(seed, n_seq=700, zero_offset_at=None):
    """Many short sequences: literal runs of 0-2 bytes (now and then 14-16),
    offsets 1-33 and a few far ones, match lengths 4-40 and 272-275.  With
    zero_offset_at=i, sequence i gets offset 0 (malformed)."""
    rng = np.random.default_rng(seed)
    block = b""
    lit = rng.integers(0, 256, 64, dtype=np.uint8).tobytes()
    out_len = 0
    for i in range(n_seq):
        if i:
            lit = rng.integers(0, 256, int(rng.choice([0] * 12 + [1, 2, 14, 15, 16])), dtype=np.uint8).tobytes()
        off = int(rng.choice(list(range(1, 34)) + [100, 1000, 5000]))
        off = min(off, out_len + len(lit))
        if i == zero_offset_at:
            off = 0
        mlen = int(rng.choice(list(range(4, 41)) + [272, 273, 274, 275]))
        block += sequence(lit, off, mlen)
        out_len += len(lit) + mlen
    return block + sequence(b"end", 0, 0)


def library(data):
    lib = L.lib()
    src = np.frombuffer(data, np.uint8)
    cap = lib.gbvr_lz4_bound(len(data))
    dst = np.zeros(cap, np.uint8)
    n = lib.gbvr_lz4_compress(src.ctypes.data, len(data), dst.ctypes.data, cap)
    assert n > 0
    return dst[:n].tobytes()


def cases():
    blocks = [
        crafted(1, [1, 2, 3, 7, 31], [4, 20, 28, 33, 100, 600, 1500], 40),
        crafted(2, [32, 33, 100, 260, 479, 480], [4, 9, 28, 29, 60, 200, 700], 80),
        crafted(3, [481, 500, 511, 512, 513, 1000, 4000], [4, 12, 30, 90, 400, 2000], 60),
        crafted(4, [1, 5, 32, 480, 481, 700, 3000], [4, 5, 31, 32, 64, 520, 3000], 120, head=3100),
        # dense: mostly 3- and 4-byte sequences, several per 32 input bytes,
        # match lengths around the one-extension-byte limits (18/19, 273/274)
        dense(12),
    ]
    rng = np.random.default_rng(9)
    x = np.arange(16384)
    datas = [bytes(16384), rng.integers(0, 256, 16384, dtype=np.uint8).tobytes(),
             np.clip(128 + 60 * np.sin(x / 300.0) + rng.normal(0, 1.5, x.size), 0, 255).astype(np.uint8).tobytes(),
             (x // 61).astype(np.uint16).tobytes()[:16384], b"lz4 brick " * 1638 + b"1234"]
    blocks += [library(d) for d in datas]
    return blocks
