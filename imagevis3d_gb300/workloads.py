"""Seeded synthetic workloads: volumes, transfer functions and cameras.

Each workload restates one benchmark configuration of the raycaster with
seeded synthetic data (no dataset files ship with the reference beyond
DemoData/c60.uvf).  Volumes come from the Philox blob generator of the
library (``gbvr_synth_params``); transfer functions and cameras are built here
on the host from ``numpy.random.default_rng(seed)``, so the GPU path and the
CPU oracle receive identical inputs.
"""
import math

import numpy as np

from .renderer import fbm_params, look_at_camera, orbit_camera, synth_params

SEED = 20261203
DIAG = math.sqrt(3.0)  # diagonal of the unit-normalised cube


def tf1d_seeded(n, seed, zero_below, value_max, points=4):
    """Piecewise-linear RGBA table of n entries through `points` seeded
    control points; alpha is 0 for data values below `zero_below`.
    Entry i corresponds to data value i * value_max / (n - 1)."""
    rng = np.random.default_rng(seed)
    xs = np.sort(rng.uniform(zero_below, value_max, points))
    cols = rng.uniform(0.0, 1.0, (points, 3))
    alphas = rng.uniform(0.15, 1.0, points)
    v = np.arange(n) * (value_max / (n - 1))
    tf = np.zeros((n, 4), np.float32)
    for c in range(3):
        tf[:, c] = np.interp(v, xs, cols[:, c])
    a = np.interp(v, np.concatenate([[zero_below], xs]), np.concatenate([[0.0], alphas]))
    a[v < zero_below] = 0.0
    tf[:, 3] = a
    return tf


def tf2d_seeded(w, h, seed, widgets=3, zero_cols=0, x_range=(0.25, 0.85)):
    """w x h RGBA table over (value, gradient magnitude) with seeded Gaussian
    ellipse widgets; row = gradient bin, column = value bin.  Alpha is the
    largest widget's Gaussian; the colour is the widgets' colours mixed by
    their Gaussians, so colour and alpha are continuous over the table (a
    colour step where the alpha is near zero would turn sub-voxel position
    differences into colour differences).  The first `zero_cols` value
    columns are transparent (empty space stays empty)."""
    rng = np.random.default_rng(seed)
    x = (np.arange(w) + 0.5) / w
    y = (np.arange(h) + 0.5) / h
    X, Y = np.meshgrid(x, y)
    tf = np.zeros((h, w, 4), np.float64)
    rgb = np.zeros((h, w, 3), np.float64)
    wsum = np.zeros((h, w), np.float64)
    for _ in range(widgets):
        cx, cy = rng.uniform(*x_range), rng.uniform(0.1, 0.6)
        sx, sy = rng.uniform(0.03, 0.12), rng.uniform(0.08, 0.3)
        col = rng.uniform(0.2, 1.0, 3)
        amax = rng.uniform(0.3, 0.9)
        g = np.exp(-0.5 * (((X - cx) / sx) ** 2 + ((Y - cy) / sy) ** 2)) * amax
        rgb += g[..., None] * col[None, None, :]
        wsum += g
        tf[..., 3] = np.maximum(tf[..., 3], g)
    tf[..., :3] = rgb / np.maximum(wsum, 1e-300)[..., None]
    tf[:, :zero_cols, 3] = 0.0
    return tf.astype(np.float32)


def orbit_views(n, width, height, elevation=20.0, radius=2.5 * DIAG, fov=45.0, start=0.0):
    """n cameras evenly spaced in azimuth, as the 360-degree capture takes
    them (ImageVis3D/UI/ImageVis3D_Capturing.cpp:170)."""
    return [orbit_camera(start + 360.0 * i / n, elevation, radius, fov, width, height) for i in range(n)]


class Workload:
    def __init__(self, name, synth, brick, tf, spv, width, height, views, lod=0,
                 value_range=None, mode=0):
        self.name = name
        self.synth = synth
        self.brick = brick
        self.tf = tf
        self.spv = spv
        self.width = width
        self.height = height
        self.views = views
        self.lod = lod
        self.value_range = value_range
        self.mode = mode


def config1(seed=SEED + 1):
    """128^3 uint8, 8 blobs (sigma 6..20, amplitude 0.3..1.0) + uniform noise
    +-4, one 128^3 brick, 256-entry TF (alpha 0 below 40), 512^2 at 45 deg,
    orbit radius 2.5 x diagonal, one seeded azimuth, 1 sample / voxel."""
    sp = synth_params((128, 128, 128), np.uint8, seed, 8, (6.0, 20.0), (0.3, 1.0), 255.0,
                      noise_kind=1, noise_amp=4.0, vmax=255.0)
    tf = tf1d_seeded(256, seed, 40.0, 255.0)
    az = float(np.random.default_rng(seed).uniform(0, 360))
    views = [orbit_camera(az, 20.0, 2.5 * DIAG, 45.0, 512, 512)]
    return Workload("c1_128cube_u8_1brick_512sq", sp, dict(brick_size=256, overlap=2), tf, 1.0,
                    512, 512, views, value_range=(0.0, 255.0))


def config2(size=1024, width=1920, height=1080, nviews=64, brick=256, seed=SEED + 2):
    """size^3 uint16 with 12-bit values: 64 blobs on a low-frequency
    background + Gaussian noise sigma 20; 256^3 bricks incl. 2 ghost voxels,
    LOD pyramid by 2x2x2 averaging; 4096-entry TF, transparent below 900 so
    background-only bricks are skipped; 1920x1080 orbit of 64
    views; 1.5 samples / voxel; finest level rendered."""
    s = size / 1024.0
    sp = synth_params((size, size, size), np.uint16, seed, 64, (24.0 * s, 90.0 * s), (0.3, 1.0),
                      2600.0, noise_kind=2, noise_amp=20.0, vmax=4095.0, bg_freq=1.0,
                      bg_level=0.15, bg_amp=0.1)
    tf = tf1d_seeded(4096, seed, 900.0, 4095.0)
    views = orbit_views(nviews, width, height)
    return Workload("c2_%dcube_u16_%dbrick_%dx%d_x%d" % (size, brick, width, height, nviews), sp,
                    dict(brick_size=brick, overlap=2), tf, 1.5, width, height, views,
                    value_range=(0.0, 4095.0))


def config3(size=2048, width=2560, height=1440, nviews=16, brick=256, seed=SEED + 3):
    """size^3 uint8 seeded fractal: 6-octave periodic value-noise fBm,
    thresholded to sparse structures (~70% of 256^3 bricks empty at 2048^3);
    2D TF 256 x 256 over (value, |gradient|) with 3 seeded Gaussian-ellipse
    widgets and Phong (1 light); isosurface mode at 3 seeded isovalues;
    2560 x 1440 orbit views, 1 sample / voxel."""
    fp = fbm_params((size, size, size), np.uint8, seed, octaves=6, base_period=2, threshold=0.58, vmax=255.0)
    tf = tf2d_seeded(256, 256, seed, widgets=3, zero_cols=8, x_range=(0.05, 0.45))
    views = orbit_views(nviews, width, height)
    isos = [float(v) for v in np.sort(np.random.default_rng(seed).uniform(12.0, 48.0, 3))]
    wl = Workload("c3_%dcube_u8_fbm_%dx%d_x%d" % (size, width, height, nviews), fp,
                  dict(brick_size=brick, overlap=2), tf, 1.0, width, height, views,
                  value_range=(0.0, 255.0), mode=1)
    wl.isovalues = isos
    return wl


# ---------------------------------------------------------------------------
# Fly-through camera path, restated from the reference's animator
# (LuaScripts/FlyThroughAnimator.lua:197-330 and 406-463): the first and last
# key points are duplicated (the non-looping preview); each segment between
# key points p1 and p2 is a cubic Bezier whose inner control points follow
# the neighbours' direction at half the segment length (computeTangents); the
# eye curve is sampled adaptively into an arc-length table (split while the
# chord and the two half chords differ by more than epsilon = linear length /
# 100000, each leaf adding its mid and end parameter); frames sit at equal arc
# length, with eye, ref and up each interpolated on their own Bezier.
# Parameters here are 0-based key indices (the script's are 1-based).
# ---------------------------------------------------------------------------
def _lerp(a, b, t):
    return a + (b - a) * t


def _decasteljau(p0, p1, p2, p3, u):
    p10, p11, p12 = _lerp(p0, p1, u), _lerp(p1, p2, u), _lerp(p2, p3, u)
    p20, p21 = _lerp(p10, p11, u), _lerp(p11, p12, u)
    p30 = _lerp(p20, p21, u)
    return p10, p20, p30, p21, p12


def _tangents(p0, p1, p2, p3):
    alpha = np.linalg.norm(p2 - p1) / 2.0
    if alpha == 0.0:
        return p1, p2
    n1 = (p2 - p0) / np.linalg.norm(p2 - p0)
    n2 = (p1 - p3) / np.linalg.norm(p1 - p3)
    return p1 + n1 * alpha, p2 + n2 * alpha


def _sample(p1, q1, q2, p2, ua, ub, eps, samples):
    # (ua, ub) are the curve parameters at the middle and at the end of this piece
    seg = _decasteljau(p1, q1, q2, p2, 0.5)
    p = seg[2]
    a, b, c = np.linalg.norm(p - p1), np.linalg.norm(p2 - p), np.linalg.norm(p2 - p1)
    if abs(c - (a + b)) > eps:
        u = (ub - ua) / 2
        _sample(p1, seg[0], seg[1], p, ua - u, ua, eps, samples)
        _sample(p, seg[3], seg[4], p2, ub - u, ub, eps, samples)
    else:
        d = samples[-1][0]
        samples.append((d + a, ua))
        samples.append((d + a + b, ub))


def arc_length_table(keys, split=100000):
    """keys: the animation's key points (already padded).  Returns the list of
    (distance, parameter) pairs."""
    eyes = [k[0] for k in keys]
    dist = sum(np.linalg.norm(eyes[i - 1] - eyes[i - 2]) for i in range(3, len(keys)))
    eps = dist / split
    samples = [(0.0, 1.0)]
    for i in range(3, len(keys)):
        q1, q2 = _tangents(eyes[i - 3], eyes[i - 2], eyes[i - 1], eyes[i])
        _sample(eyes[i - 2], q1, q2, eyes[i - 1], i - 1.5, i - 1.0, eps, samples)
    return samples


def _camera_at(keys, table, s):
    idx = 1
    while table[idx][0] < s:
        idx += 1
    (d0, u0), (d1, u1) = table[idx - 1], table[idx]
    u = u0 + (s - d0) / (d1 - d0) * (u1 - u0) if d1 != d0 else u0
    i = int(np.floor(u))
    w = u - i
    if w == 0.0:
        return keys[i]
    cam = []
    for c in range(3):
        q1, q2 = _tangents(keys[i - 1][c], keys[i][c], keys[i + 1][c], keys[i + 2][c])
        cam.append(_decasteljau(keys[i][c], q1, q2, keys[i + 1][c], w)[2])
    return tuple(cam)


def flythrough(keys, frames):
    """keys: list of (eye, ref, up) key points (at least two); returns `frames`
    (eye, ref, up) triples at equal arc length from the first key to the last."""
    keys = [tuple(np.asarray(k, np.float64) for k in key) for key in keys]
    keys = [keys[0]] + keys + [keys[-1]]
    table = arc_length_table(keys)
    total = table[-1][0]
    return [_camera_at(keys, table, min(total * f / max(frames - 1, 1), total)) for f in range(frames)]


def flythrough_views(keys, frames, width, height, fov=45.0, znear=0.01, zfar=10.0):
    return [look_at_camera(e, r, u, fov, width, height, znear, zfar) for e, r, u in flythrough(keys, frames)]


def config4(size=(8192, 8192, 4096), width=1920, height=1080, frames=120, brick=256, lods=6, seed=SEED + 4):
    """Out-of-core volume: layered seeded blobs, 192 of them over a
    low-frequency background layer (no per-voxel noise), uint8, 256^3 bricks
    with 2 ghosts and `lods` levels, a fly-through of `frames` frames at
    width x height (from outside the volume into it and through), 1D TF with
    256 entries (alpha 0 below 60)."""
    n = max(size)
    sp = synth_params(size, np.uint8, seed, 192, (0.01 * n, 0.04 * n), (0.3, 1.0), 255.0, vmax=255.0,
                      bg_freq=1.5, bg_level=0.08, bg_amp=0.1)
    tf = tf1d_seeded(256, seed, 60.0, 255.0)
    m = [s / n for s in size]  # normalised half extents are m / 2
    keys = [((-0.9 * m[0], 0.1, -0.6 * m[2]), (0.0, 0.0, 0.0), (0, 1, 0)),
            ((-0.45 * m[0], 0.05, -0.35 * m[2]), (0.1, 0.0, 0.1), (0, 1, 0)),
            ((0.0, -0.05, -0.25 * m[2]), (0.2, -0.05, 0.3), (0, 1, 0)),
            ((0.35 * m[0], 0.0, 0.0), (0.0, 0.0, 0.35 * m[2]), (0, 1, 0)),
            ((0.3 * m[0], 0.05, 0.35 * m[2]), (-0.2, 0.0, 0.2), (0, 1, 0)),
            ((-0.1 * m[0], 0.1, 0.45 * m[2]), (-0.35, 0.0, 0.0), (0, 1, 0)),
            ((-0.5 * m[0], 0.1, 0.2 * m[2]), (-0.2, 0.0, -0.3), (0, 1, 0))]
    views = flythrough_views(keys, frames, width, height)
    wl = Workload("c4_%dx%dx%d_u8_ooc_%dx%d_x%d" % (size[0], size[1], size[2], width, height, frames), sp,
                  dict(brick_size=brick, overlap=2, max_lods=lods), tf, 1.0, width, height, views,
                  value_range=(0.0, 255.0))
    wl.keys = keys
    return wl
