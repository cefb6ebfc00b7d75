"""Generate the c60 golden fixture from the reference's own demo dataset.

Reads ``DemoData/c60.uvf``, ``DemoData/c60.1dt`` and ``DemoData/c60.2dt`` from the
reference tree (path given on the command line or in IMAGEVIS3D_REFERENCE) and
writes ``c60.npz`` beside this script.  The fixture holds what the reference's
UVF writer stored: the 128^3 uint8 voxels, the 256-bin 1D histogram, the
256x256 2D histogram with its float32 max-gradient, the min/max block, the
global-header checksum and every header field needed to re-emit the file byte
for byte.  Tests use it on machines where the reference tree is absent.

Usage: python tests/golden/make_c60_golden.py [REFERENCE_ROOT]
(REFERENCE_ROOT: an ImageVis3D source tree; default: $IMAGEVIS3D_REFERENCE)
"""
import hashlib
import os
import struct
import sys

import numpy as np


def u64(buf, off):
    return struct.unpack_from("<Q", buf, off)[0]


def parse_blocks(f):
    assert f[:8] == b"UVF-DATA"
    p = 9
    version, cs_sem, cs_len = struct.unpack_from("<3Q", f, p)
    p += 24
    checksum = f[p:p + cs_len]
    p += cs_len
    addl = u64(f, p)
    p += 8 + addl
    blocks = []
    while True:
        start = p
        slen = u64(f, p)
        bid = f[p + 8:p + 8 + slen].decode("ascii")
        q = p + 8 + slen
        sem, comp, nxt = struct.unpack_from("<3Q", f, q)
        blocks.append(dict(start=start, id=bid, sem=sem, comp=comp, next=nxt,
                           payload=q + 24))
        if nxt == 0:
            break
        p = start + nxt
    return dict(version=version, cs_sem=cs_sem, checksum=checksum, blocks=blocks)


def parse_1dt(text):
    tok = text.split()
    n = int(tok[0])
    return np.array(tok[1:1 + 4 * n], dtype=np.float32).reshape(n, 4)


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("IMAGEVIS3D_REFERENCE", "")
    if not root:
        sys.exit("usage: make_c60_golden.py REFERENCE_ROOT (or set IMAGEVIS3D_REFERENCE)")
    demo = os.path.join(root, "DemoData")
    f = open(os.path.join(demo, "c60.uvf"), "rb").read()
    info = parse_blocks(f)
    by_sem = {b["sem"]: b for b in info["blocks"]}

    rast = by_sem[1]
    w = struct.unpack_from("<41Q", f, rast["payload"])
    dims = w[20:23]
    data_off = rast["payload"] + 41 * 8 + 1 + 8
    vol = np.frombuffer(f, np.uint8, dims[0] * dims[1] * dims[2], data_off)
    vol = vol.reshape(dims[2], dims[1], dims[0])

    h1 = by_sem[5]
    n1 = u64(f, h1["payload"])
    hist1d = np.frombuffer(f, "<u8", n1, h1["payload"] + 8).astype(np.uint64)

    h2 = by_sem[6]
    maxgrad = struct.unpack_from("<f", f, h2["payload"])[0]
    nx, ny = struct.unpack_from("<2Q", f, h2["payload"] + 4)
    hist2d = np.frombuffer(f, "<u8", nx * ny, h2["payload"] + 20).astype(np.uint64)
    hist2d = hist2d.reshape(nx, ny)

    mm = by_sem[7]
    nbricks, ncomp = struct.unpack_from("<2Q", f, mm["payload"])
    minmax = np.frombuffer(f, "<f8", 4 * nbricks * ncomp, mm["payload"] + 16)

    tf1d = parse_1dt(open(os.path.join(demo, "c60.1dt")).read())
    tf2d_text = open(os.path.join(demo, "c60.2dt")).read()

    np.savez_compressed(
        os.path.join(os.path.dirname(os.path.abspath(__file__)), "c60.npz"),
        volume=vol,
        hist1d=hist1d,
        hist2d=hist2d,
        maxgrad_f32=np.array([maxgrad], np.float32),
        minmax=minmax.copy(),
        raster_words=np.array(w, np.uint64),
        block_ids=np.array([b["id"] for b in info["blocks"]]),
        block_sems=np.array([b["sem"] for b in info["blocks"]], np.uint64),
        block_starts=np.array([b["start"] for b in info["blocks"]], np.uint64),
        checksum=np.frombuffer(info["checksum"], np.uint8),
        file_md5=np.frombuffer(hashlib.md5(f).digest(), np.uint8),
        file_size=np.array([len(f)], np.uint64),
        tf1d=tf1d,
        tf2d_text=np.array([tf2d_text]),
    )
    print("wrote c60.npz: dims", dims, "hist1d", n1, "hist2d", (nx, ny),
          "maxgrad", maxgrad)


if __name__ == "__main__":
    main()
