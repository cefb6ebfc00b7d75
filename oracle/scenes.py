"""Benchmark scenes restated on the CPU side: volume parameters, seeded
transfer functions and cameras of the raycast workloads.

TEST INFRASTRUCTURE ONLY, like the rest of oracle/: bench.py's reference arm
renders from these without loading the GPU library, and the tests check that
they equal the library's own workloads (imagevis3d_gb300.workloads).  The
cameras come from the oracle's FP64 camera code (orc.orbit_camera), not the
library's; the volume parameters are the seeded blob generator's
(gbvr_synth_params), float fields rounded to float32 as the library stores
them; the transfer-function rule is the one the workloads state.
"""
import math
from types import SimpleNamespace

import numpy as np

from . import orc

SEED = 20261203
DIAG = math.sqrt(3.0)


def _f32(x):
    return float(np.float32(x))


def blob_params(dims, dtype, seed, nblobs, sigma, amp, scale, noise_kind=0, noise_amp=0.0, vmax=255.0,
                bg_freq=0.0, bg_level=0.0, bg_amp=0.0):
    """The blob generator's parameters (dtype 0 u8, 1 u16, 2 f32)."""
    return SimpleNamespace(dims=[int(d) for d in dims], dtype=int(dtype), seed=int(seed), nblobs=int(nblobs),
                           sigma_lo=_f32(sigma[0]), sigma_hi=_f32(sigma[1]), amp_lo=_f32(amp[0]),
                           amp_hi=_f32(amp[1]), bg_freq=_f32(bg_freq), bg_level=_f32(bg_level),
                           bg_amp=_f32(bg_amp), scale=_f32(scale), noise_kind=int(noise_kind),
                           noise_amp=_f32(noise_amp), vmax=_f32(vmax))


def tf1d_seeded(n, seed, zero_below, value_max, points=4):
    """n RGBA entries, piecewise linear through `points` seeded control
    points (colours uniform in [0, 1], alphas in [0.15, 1]); alpha 0 below
    `zero_below`; entry i is data value i * value_max / (n - 1)."""
    rng = np.random.default_rng(seed)
    knots = np.sort(rng.uniform(zero_below, value_max, points))
    rgb = rng.uniform(0.0, 1.0, (points, 3))
    alpha = rng.uniform(0.15, 1.0, points)
    value = np.arange(n) * (value_max / (n - 1))
    out = np.zeros((n, 4), np.float32)
    for c in range(3):
        out[:, c] = np.interp(value, knots, rgb[:, c])
    a = np.interp(value, np.concatenate([[zero_below], knots]), np.concatenate([[0.0], alpha]))
    a[value < zero_below] = 0.0
    out[:, 3] = a
    return out


def orbit_views(n, width, height, elevation=20.0, radius=2.5 * DIAG, fov=45.0, start=0.0):
    """n orbit cameras evenly spaced in azimuth (FP64 oracle cameras)."""
    return [orc.orbit_camera(start + 360.0 * i / n, elevation, radius, fov, width, height) for i in range(n)]


def config2(size=1024, width=1920, height=1080, nviews=64, brick=256, seed=SEED + 2):
    """The 1024^3 uint16 orbit workload: 12-bit values from 64 blobs on a
    low-frequency background plus Gaussian noise sigma 20, 4096-entry TF
    transparent below 900, 1.5 samples per voxel, 64 views at 1920x1080."""
    s = size / 1024.0
    synth = blob_params((size, size, size), 1, seed, 64, (24.0 * s, 90.0 * s), (0.3, 1.0), 2600.0, noise_kind=2,
                        noise_amp=20.0, vmax=4095.0, bg_freq=1.0, bg_level=0.15, bg_amp=0.1)
    return SimpleNamespace(name="c2_%dcube_u16_%dbrick_%dx%d_x%d" % (size, brick, width, height, nviews),
                           synth=synth, tf=tf1d_seeded(4096, seed, 900.0, 4095.0), spv=1.5, width=width,
                           height=height, views=orbit_views(nviews, width, height), value_range=(0.0, 4095.0))
