"""The CPU side's scenes (oracle/scenes.py) against the library's workloads,
and the reference arm of bench.py running without the GPU library.

The oracle computes its cameras with its own FP64 camera code, so this is
also the independent check of the library's camera matrices that every
parity test relies on."""
import json
import os
import subprocess
import sys

import numpy as np

from conftest import ROOT


def test_c2_scene_equals_library_workload(orc):
    from oracle import scenes
    from imagevis3d_gb300 import workloads
    a = scenes.config2(size=64, nviews=16)
    b = workloads.config2(size=64, nviews=16)
    assert a.name == b.name
    for f in ("sigma_lo", "sigma_hi", "amp_lo", "amp_hi", "bg_freq", "bg_level", "bg_amp", "scale", "noise_amp",
              "vmax", "seed", "nblobs", "noise_kind", "dtype"):
        assert getattr(a.synth, f) == getattr(b.synth, f), f
    assert list(a.synth.dims) == [b.synth.dims[i] for i in range(3)]
    assert np.array_equal(a.tf, b.tf)
    assert (a.spv, a.width, a.height, tuple(a.value_range)) == (b.spv, b.width, b.height, tuple(b.value_range))
    # cameras: FP64 in both, rounded to float32 once; equal within float32 rounding
    for (v1, p1), (v2, p2) in zip(a.views, b.views):
        assert np.allclose(v1, v2, rtol=2e-7, atol=2e-7)
        assert np.allclose(p1, p2, rtol=2e-7, atol=2e-7)
    # the same volume from both parameter sets
    assert np.array_equal(orc.synth_blobs(a.synth), orc.synth_blobs(b.synth))


def test_look_at_camera_equals_library():
    from oracle import orc
    from imagevis3d_gb300 import look_at_camera
    rng = np.random.default_rng(5)
    for _ in range(20):
        eye = rng.uniform(-3, 3, 3)
        ref = rng.uniform(-0.5, 0.5, 3)
        v1, p1 = orc.look_at_camera(eye, ref, (0, 1, 0), 40.0, 0.05, 9.0, 640, 360)
        v2, p2 = look_at_camera(eye, ref, (0, 1, 0), 40.0, 640, 360, znear=0.05, zfar=9.0)
        assert np.allclose(v1, v2, rtol=2e-7, atol=2e-7)
        assert np.allclose(p1, p2, rtol=2e-7, atol=2e-7)


def test_reference_arm_runs_without_the_library():
    """bench.py --impl reference on a small volume: one JSON line, and neither
    the package nor libgbvr.so is in the process."""
    code = ("import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--size', '64', '--steps', '1', "
            "'--warmup', '3', '--ref-seconds', '0.3']; import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print('LOADED', int('imagevis3d_gb300' in sys.modules), int('libgbvr' in maps))")
    p = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    lines = p.stdout.strip().splitlines()
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["value"] > 0 and rec["cpu_baseline"]["kind"] == "port"
    assert lines[-1] == "LOADED 0 0"


def test_procedural_fbm_render_equals_flat_volume_render(orc):
    """The oracle's on-demand fractal voxels give the same FP64 image as the
    generated volume, in every mode that reads voxels differently."""
    from imagevis3d_gb300 import workloads
    wl = workloads.config3(size=48, width=40, height=30, nviews=2)
    vol = orc.synth_fbm(wl.synth)
    proc = orc.ProceduralFbm(wl.synth)
    v, p = workloads.orbit_views(1, 40, 30, radius=1.5 * workloads.DIAG, start=30.0)[0]
    for kw in (dict(mode=1, grad_max=0.02), dict(mode=2, iso=20.0), dict(mode=0, interp=0)):
        tf = wl.tf if kw["mode"] == 1 else np.tile(np.float32([[0.5, 0.6, 0.7, 0.05]]), (256, 1))
        a, na = orc.render(vol, v, p, 40, 30, tf, value_range=wl.value_range, **kw)
        b, nb = orc.render(proc, v, p, 40, 30, tf, value_range=wl.value_range, **kw)
        assert np.array_equal(a, b) and na == nb
