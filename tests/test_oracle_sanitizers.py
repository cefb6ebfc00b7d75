"""The CPU oracle itself under AddressSanitizer and UndefinedBehaviorSanitizer:
every render mode (1D and 2D TF, isosurface, MIP), the clip plane, bounding
boxes, ClearView, slices, LOD averaging and the histograms, on small seeded
volumes.  The oracle is the checker of every parity test, so it must be free
of out-of-bounds reads and undefined behaviour itself.  No GPU."""
import os
import shutil
import subprocess
import sys
import textwrap

import pytest

from tests.conftest import ROOT

SCRIPT = textwrap.dedent("""
    import ctypes as C, sys
    sys.path.insert(0, ROOT)
    import numpy as np
    from oracle import orc
    from imagevis3d_gb300 import synth_params, orbit_camera, workloads
    L = C.CDLL(LIB)
    L.orc_render.restype = C.c_int64
    L.orc_hist1d.restype = C.c_int64
    L.orc_hist2d.restype = C.c_double
    L.orc_lod_dims.restype = C.c_int
    L.orc_max_threads.restype = C.c_int
    orc._lib = L
    view, proj = orbit_camera(30, 20, 2.5 * workloads.DIAG, 45, 41, 33)
    for dt, vmax in ((np.uint8, 255.0), (np.uint16, 4095.0)):
        sp = synth_params((37, 29, 23), dt, 5, 6, (3.0, 8.0), (0.3, 1.0), vmax * 0.7, noise_kind=1,
                          noise_amp=3.0, vmax=vmax)
        vol = orc.synth_blobs(sp)
        tf = workloads.tf1d_seeded(256, 3, vmax * 0.2, vmax)
        rng = (0.0, vmax)
        for mode in (0, 2, 3):
            orc.render(vol, view, proj, 41, 33, tf, value_range=rng, mode=mode, iso=vmax * 0.4)
        orc.render(vol, view, proj, 41, 33, workloads.tf2d_seeded(64, 32, 3), value_range=rng, mode=1,
                   grad_max=0.2)
        orc.render(vol, view, proj, 41, 33, tf, value_range=rng, clip=(1.0, 0.2, 0.0, 0.05))
        orc.render(vol, view, proj, 41, 33, tf, value_range=rng,
                   bbox=dict(global_=True, local=True, interior=12, rgb=((1, 0, 0), (0, 1, 0))))
        orc.render(vol, view, proj, 41, 33, tf, value_range=rng, mode=2, iso=vmax * 0.3,
                   cv=dict(iso=vmax * 0.5, rgb=(1, 0, 0), context=1.0, border=1.0, focus=(20, 16), radius=10.0))
        for axis in range(3):
            orc.render_slice(vol, axis, 10, 41, 33, tf, value_range=rng, mip=axis == 1)
        orc.downsample(vol)
        h1 = orc.hist1d(vol)
        orc.hist2d(vol, vmax, len(h1))
    print("oracle ok")
""")


def test_oracle_under_sanitizers(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    runtimes = []
    for name in ("libasan.so", "libubsan.so"):
        p = subprocess.run(["g++", "-print-file-name=" + name], capture_output=True, text=True).stdout.strip()
        if not os.path.isabs(p) or not os.path.exists(p):
            pytest.skip("sanitizer runtime %s not available" % name)
        runtimes.append(p)
    lib = str(tmp_path / "liborc_san.so")
    r = subprocess.run(["g++", "-O1", "-g", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                        "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
                        os.path.join(ROOT, "oracle", "oracle.cpp"), "-o", lib], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, LD_PRELOAD=":".join(runtimes), ASAN_OPTIONS="detect_leaks=0")
    code = "ROOT = %r\nLIB = %r\n" % (ROOT, lib) + SCRIPT
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0 and "oracle ok" in r.stdout, (r.stdout + r.stderr)[-4000:]
