"""ctypes binding of the CPU oracle (oracle/liborc.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg, never by the product.  See oracle.cpp for the
rules it restates and the reference files they come from.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

I64 = C.c_int64
D = C.c_double
U64P = C.POINTER(C.c_uint64)
_DT = {np.dtype(np.uint8): 0, np.dtype(np.uint16): 1, np.dtype(np.float32): 2}


class RenderParams(C.Structure):
    _fields_ = [
        ("vol", C.c_void_p), ("dtype", C.c_int), ("dims", I64 * 3), ("extent", D * 3),
        ("tf", C.POINTER(C.c_float)), ("tf_w", C.c_int), ("tf_h", C.c_int), ("mode", C.c_int),
        ("interp", C.c_int), ("value_lo", D), ("value_hi", D), ("grad_max", D),
        ("samples_per_voxel", D), ("ert", D), ("iso", D), ("iso_rgb", D * 3), ("lighting", C.c_int),
        ("amb", D * 3), ("diff", D * 3), ("spec", D * 3), ("shininess", D),
        ("light_dir_eye", D * 3), ("bg", D * 3), ("inv_viewproj", D * 16), ("inv_view", D * 16),
        ("width", C.c_int), ("height", C.c_int), ("clip_on", C.c_int), ("clip", D * 4),
        ("bbox_global", C.c_int), ("bbox_local", C.c_int), ("line_rgb", D * 6), ("view", D * 16),
        ("proj", D * 16), ("brick_interior", I64), ("line_keys", C.c_void_p),
        ("cv_on", C.c_int), ("cv_iso", D), ("cv_rgb", D * 3), ("cv_context", D), ("cv_border", D),
        ("cv_focus", D * 2), ("cv_radius", D),
        ("bg_grad", C.c_int), ("bg_top", D * 3),
        ("proc_fbm", C.c_int), ("fbm_seed", C.c_uint32), ("fbm_octaves", C.c_int), ("fbm_base_period", C.c_int),
        ("fbm_threshold", C.c_float), ("fbm_vmax", C.c_float),
    ]


class BlobTables(C.Structure):
    _fields_ = [
        ("nblobs", C.c_int), ("amp", C.c_void_p), ("ex", C.c_void_p), ("ey", C.c_void_p),
        ("ez", C.c_void_p), ("bgx", C.c_void_p), ("bgy", C.c_void_p), ("bgz", C.c_void_p),
        ("bg_level", C.c_float), ("bg_amp", C.c_float), ("scale", C.c_float),
        ("noise_amp", C.c_float), ("noise_kind", C.c_int), ("vmax", C.c_float),
        ("seed", C.c_uint32),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        _lib.orc_render.restype = I64
        _lib.orc_hist1d.restype = I64
        _lib.orc_hist2d.restype = D
        _lib.orc_lod_dims.restype = C.c_int
        _lib.orc_max_threads.restype = C.c_int
    return _lib


def _dims(vol):
    return (I64 * 3)(vol.shape[2], vol.shape[1], vol.shape[0])


def lod_dims(dims, brick, ghost, max_lods=0):
    out = (I64 * 96)()
    n = lib().orc_lod_dims((I64 * 3)(*dims), brick, ghost, max_lods, out)
    return [tuple(out[3 * i:3 * i + 3]) for i in range(n)]


def brick_grid(dims, brick, ghost):
    nb = (I64 * 3)()
    interior = I64()
    lib().orc_brick_grid((I64 * 3)(*dims), brick, ghost, nb, C.byref(interior))
    return tuple(nb), interior.value


def extract_brick(vol, brick, ghost, b):
    dims = (vol.shape[2], vol.shape[1], vol.shape[0])
    o = (I64 * 3)()
    s = (I64 * 3)()
    lib().orc_brick_extent((I64 * 3)(*dims), brick, ghost, (I64 * 3)(*b), o, s)
    out = np.empty((s[2], s[1], s[0]), vol.dtype)
    vol = np.ascontiguousarray(vol)
    lib().orc_extract_brick(vol.ctypes.data_as(C.c_void_p), _DT[vol.dtype], _dims(vol), brick, ghost,
                            (I64 * 3)(*b), out.ctypes.data_as(C.c_void_p))
    return out, tuple(o)


def downsample(vol):
    vol = np.ascontiguousarray(vol)
    out = np.empty(((vol.shape[0] + 1) // 2, (vol.shape[1] + 1) // 2, (vol.shape[2] + 1) // 2), vol.dtype)
    lib().orc_downsample(vol.ctypes.data_as(C.c_void_p), _DT[vol.dtype], _dims(vol),
                         out.ctypes.data_as(C.c_void_p))
    return out


def hist1d(vol, max_bins=4096):
    vol = np.ascontiguousarray(vol)
    out = np.zeros(65536, np.uint64)
    f = I64()
    n = lib().orc_hist1d(vol.ctypes.data_as(C.c_void_p), _DT[vol.dtype], I64(vol.size), max_bins,
                         out.ctypes.data_as(U64P), C.byref(f))
    return out[:n].copy(), f.value


def hist2d(vol, max_scalar, nx, merge=1):
    vol = np.ascontiguousarray(vol)
    out = np.zeros(nx * 256, np.uint64)
    mg = lib().orc_hist2d(vol.ctypes.data_as(C.c_void_p), _DT[vol.dtype], _dims(vol), D(max_scalar),
                          I64(nx), I64(merge), out.ctypes.data_as(U64P))
    return out.reshape(nx, 256), mg


def synth_blobs(params):
    """CPU restatement of the seeded blob generator (gbvr_synth_params)."""
    dims = [params.dims[i] for i in range(3)]
    nb = params.nblobs
    amp = np.zeros(max(nb, 1), np.float32)
    ex = np.zeros(max(nb * dims[0], 1), np.float32)
    ey = np.zeros(max(nb * dims[1], 1), np.float32)
    ez = np.zeros(max(nb * dims[2], 1), np.float32)
    bgx = np.zeros(dims[0], np.float32)
    bgy = np.zeros(dims[1], np.float32)
    bgz = np.zeros(dims[2], np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    lib().orc_blob_tables_make((I64 * 3)(*dims), C.c_uint32(params.seed), nb, D(params.sigma_lo),
                               D(params.sigma_hi), D(params.amp_lo), D(params.amp_hi),
                               D(params.bg_freq), fp(amp), fp(ex), fp(ey), fp(ez), fp(bgx), fp(bgy),
                               fp(bgz))
    t = BlobTables()
    t.nblobs = nb
    t.amp, t.ex, t.ey, t.ez = (a.ctypes.data for a in (amp, ex, ey, ez))
    bg = params.bg_freq > 0
    t.bgx = bgx.ctypes.data if bg else None
    t.bgy = bgy.ctypes.data if bg else None
    t.bgz = bgz.ctypes.data if bg else None
    t.bg_level, t.bg_amp, t.scale = params.bg_level, params.bg_amp, params.scale
    t.noise_amp, t.noise_kind, t.vmax, t.seed = params.noise_amp, params.noise_kind, params.vmax, params.seed
    dt = {0: np.uint8, 1: np.uint16, 2: np.float32}[params.dtype]
    out = np.empty((dims[2], dims[1], dims[0]), dt)
    keep = (amp, ex, ey, ez, bgx, bgy, bgz)  # noqa: F841  (alive during the call)
    lib().orc_synth_blobs(C.byref(t), (I64 * 3)(*dims), params.dtype, out.ctypes.data_as(C.c_void_p))
    return out


class ProceduralFbm:
    """The seeded fractal volume (gbvr_fbm_params) as a render input whose
    voxels the oracle evaluates where its samples need them."""

    def __init__(self, params):
        self.dims = [int(params.dims[i]) for i in range(3)]
        self.dtype = int(params.dtype)
        self.seed = int(params.seed)
        self.octaves = int(params.octaves)
        self.base_period = int(params.base_period)
        self.threshold = float(np.float32(params.threshold))
        self.vmax = float(np.float32(params.vmax))


def render(vol, view, proj, width, height, tf, spv=1.0, value_range=(0.0, 255.0), mode=0,
           interp=1, ert=0.99, extent=None, grad_max=1.0, iso=0.0, iso_rgb=(1, 1, 1), lighting=1,
           amb=(0.1, 0.1, 0.1), diff=(1, 1, 1), spec=(1, 1, 1), shininess=8.0,
           light_dir=(0, 0, -1), bg=(0, 0, 0), pixels=None, threads=0, clip=None, bbox=None, cv=None,
           bg_top=None):
    """FP64 render of `vol` (the flat level, (z, y, x)), or of a procedural
    fractal volume when `vol` is a ProceduralFbm (voxels evaluated on demand,
    for volumes too large for host memory).  mode 0 1D TF, 1 2D TF
    + Phong, 2 isosurface, 3 maximum-intensity projection; clip = plane
    (a, b, c, d) dropping samples with a x + b y + c z + d > 0; bbox = dict
    (global_, local, interior = brick edge minus two ghosts, rgb = (global,
    local) colours) for bounding-box lines; cv = dict(iso, rgb, context,
    border, focus = (x, y) pixels, radius pixels) for ClearView (mode 2);
    bg_top: the top edge's background colour (a vertical gradient down to
    `bg`, as setBGColors draws two colours).
    Returns (rgba float64 [n, 4] or [h, w, 4], samples)."""
    tf = np.ascontiguousarray(tf, np.float32)
    p = RenderParams()
    if isinstance(vol, ProceduralFbm):
        shape = (vol.dims[2], vol.dims[1], vol.dims[0])
        p.vol = None
        p.dtype = vol.dtype
        p.proc_fbm, p.fbm_seed, p.fbm_octaves, p.fbm_base_period = 1, vol.seed, vol.octaves, vol.base_period
        p.fbm_threshold, p.fbm_vmax = vol.threshold, vol.vmax
    else:
        vol = np.ascontiguousarray(vol)
        shape = vol.shape
        p.vol = vol.ctypes.data
        p.dtype = _DT[vol.dtype]
    for i, d in enumerate((shape[2], shape[1], shape[0])):
        p.dims[i] = d
    if bg_top is not None:
        p.bg_grad = 1
        for i in range(3):
            p.bg_top[i] = bg_top[i]
    if extent is None:
        m = max(shape)
        extent = (shape[2] / m, shape[1] / m, shape[0] / m)
    for i in range(3):
        p.extent[i] = extent[i]
    p.tf = tf.ctypes.data_as(C.POINTER(C.c_float))
    if tf.ndim == 2:
        p.tf_w, p.tf_h = tf.shape[0], 1
    else:
        p.tf_w, p.tf_h = tf.shape[1], tf.shape[0]
    p.mode, p.interp = mode, interp
    p.value_lo, p.value_hi = value_range
    p.grad_max = grad_max
    p.samples_per_voxel, p.ert, p.iso = spv, ert, iso
    p.lighting = lighting
    for i in range(3):
        p.iso_rgb[i], p.amb[i], p.diff[i], p.spec[i] = iso_rgb[i], amb[i], diff[i], spec[i]
        p.light_dir_eye[i], p.bg[i] = light_dir[i], bg[i]
    p.shininess = shininess
    V = np.asarray(view, np.float64).reshape(4, 4)
    Pm = np.asarray(proj, np.float64).reshape(4, 4)
    Mi = np.linalg.inv(Pm @ V)
    Vi = np.linalg.inv(V)
    for i in range(16):
        p.inv_viewproj[i] = Mi.ravel()[i]
        p.inv_view[i] = Vi.ravel()[i]
    p.width, p.height = width, height
    if clip is not None:
        p.clip_on = 1
        for i in range(4):
            p.clip[i] = clip[i]
    _set_lines(p, view, proj, bbox)
    if cv:
        p.cv_on = 1
        p.cv_iso = cv["iso"]
        for k in range(3):
            p.cv_rgb[k] = float(np.float32(cv.get("rgb", (1, 1, 1))[k]))
        p.cv_context = float(np.float32(cv.get("context", 1.0)))
        p.cv_border = float(np.float32(cv.get("border", 1.0)))
        p.cv_focus[0], p.cv_focus[1] = (float(np.float32(x)) for x in cv["focus"])
        p.cv_radius = float(np.float32(cv["radius"]))
    if pixels is None:
        out = np.zeros((height * width, 4), np.float64)
        ns = lib().orc_render(C.byref(p), None, I64(0), out.ctypes.data_as(C.POINTER(D)), threads)
        return out.reshape(height, width, 4), ns
    pix = np.ascontiguousarray(pixels, np.int64)
    out = np.zeros((pix.size, 4), np.float64)
    ns = lib().orc_render(C.byref(p), pix.ctypes.data_as(C.POINTER(I64)), I64(pix.size),
                          out.ctypes.data_as(C.POINTER(D)), threads)
    return out, ns


def _set_lines(p, view, proj, bbox):
    if not bbox:
        return
    p.bbox_global = 1 if bbox.get("global_") else 0
    p.bbox_local = 1 if bbox.get("local") else 0
    rgb = bbox.get("rgb", ((1.0, 1.0, 1.0), (0.6, 0.6, 0.6)))
    for c in range(2):
        for k in range(3):
            p.line_rgb[3 * c + k] = float(np.float32(rgb[c][k]))
    v32 = np.asarray(view, np.float32).ravel()
    p32 = np.asarray(proj, np.float32).ravel()
    for i in range(16):
        p.view[i] = float(v32[i])
        p.proj[i] = float(p32[i])
    p.brick_interior = int(bbox.get("interior", 1 << 40))


def line_keys(dims, extent, view, proj, width, height, bbox):
    """Per-pixel keys of the nearest bounding-box line ([h, w] uint32,
    0xffffffff where none) for a level of `dims` (x, y, z)."""
    p = RenderParams()
    for i in range(3):
        p.dims[i] = dims[i]
        p.extent[i] = extent[i]
    p.width, p.height = width, height
    _set_lines(p, view, proj, bbox)
    out = np.empty((height, width), np.uint32)
    lib().orc_line_keys(C.byref(p), out.ctypes.data_as(C.c_void_p))
    return out


def lz4_decompress(block, out_n):
    """Oracle LZ4 block decoder: bytes, or None when malformed."""
    src = np.frombuffer(bytes(block), np.uint8) if len(block) else np.zeros(1, np.uint8)
    out = np.zeros(max(out_n, 1), np.uint8)
    f = lib().orc_lz4_decompress
    f.restype = I64
    n = f(src.ctypes.data_as(C.c_void_p), I64(len(block)), out.ctypes.data_as(C.c_void_p), I64(out_n))
    return None if n < 0 else out[:n].tobytes()


def render_slice(vol, axis, coord, width, height, tf, value_range=(0.0, 255.0), flip_x=False, flip_y=False,
                 mip=False, interp=1, extent=None, bg=(0, 0, 0), bg_top=None):
    """FP64 2D slice view of the flat level `vol` ((z, y, x)): [h, w, 4];
    bg_top: the top edge's background colour of a vertical gradient."""
    vol = np.ascontiguousarray(vol)
    tf = np.ascontiguousarray(tf, np.float32)
    p = RenderParams()
    p.vol = vol.ctypes.data
    p.dtype = _DT[vol.dtype]
    for i, d in enumerate((vol.shape[2], vol.shape[1], vol.shape[0])):
        p.dims[i] = d
    if extent is None:
        m = max(vol.shape)
        extent = (vol.shape[2] / m, vol.shape[1] / m, vol.shape[0] / m)
    for i in range(3):
        p.extent[i] = extent[i]
        p.bg[i] = bg[i]
    if bg_top is not None:
        p.bg_grad = 1
        for i in range(3):
            p.bg_top[i] = bg_top[i]
    p.tf = tf.ctypes.data_as(C.POINTER(C.c_float))
    p.tf_w, p.tf_h = tf.shape[0], 1
    p.interp = interp
    p.value_lo, p.value_hi = value_range
    p.width, p.height = width, height
    out = np.zeros((height, width, 4), np.float64)
    lib().orc_render_slice(C.byref(p), axis, D(coord), int(flip_x), int(flip_y), int(mip),
                           out.ctypes.data_as(C.POINTER(D)))
    return out


def max_threads():
    return lib().orc_max_threads()


def uvf_build_timed(vol, brick=256, ghost=2, threads=0):
    """The CPU UVF build of `vol` on `threads` threads (0 = all): returns
    (total seconds, {pyramid, bricks, hist1d, hist2d} seconds)."""
    vol = np.ascontiguousarray(vol)
    ph = (D * 4)()
    lib().orc_uvf_build_timed.restype = D
    t = lib().orc_uvf_build_timed(vol.ctypes.data_as(C.c_void_p), _DT[vol.dtype], _dims(vol), int(brick),
                                  int(ghost), int(threads), ph)
    return t, dict(zip(("pyramid", "bricks", "hist1d", "hist2d"), list(ph)))


def orbit_camera(azimuth_deg, elevation_deg, radius, fov_deg, width, height):
    """FP64 orbit camera (orc_orbit_camera), rounded to float32 row-major
    (view, proj) as the library takes them.  The angles, radius and field of
    view are float32 numbers, as the library's camera call receives them."""
    v = np.zeros(16, np.float32)
    p = np.zeros(16, np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    f32 = lambda x: D(float(np.float32(x)))
    lib().orc_orbit_camera(f32(azimuth_deg), f32(elevation_deg), f32(radius), f32(fov_deg), int(width), int(height),
                           fp(v), fp(p))
    return v.reshape(4, 4), p.reshape(4, 4)


def look_at_camera(eye, ref, up, fov_deg, znear, zfar, width, height):
    """FP64 look-at camera (orc_look_at_camera), rounded to float32; inputs
    are float32 numbers, as the library's camera call receives them."""
    v = np.zeros(16, np.float32)
    p = np.zeros(16, np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    f32 = lambda x: D(float(np.float32(x)))
    d3 = lambda a: (D * 3)(*[float(np.float32(x)) for x in a])
    lib().orc_look_at_camera(d3(eye), d3(ref), d3(up), f32(fov_deg), f32(znear), f32(zfar), int(width), int(height),
                             fp(v), fp(p))
    return v.reshape(4, 4), p.reshape(4, 4)


def synth_fbm(params):
    """CPU restatement of the seeded fractal generator (gbvr_fbm_params)."""
    dims = [params.dims[i] for i in range(3)]
    dt = {0: np.uint8, 1: np.uint16, 2: np.float32}[params.dtype]
    out = np.empty((dims[2], dims[1], dims[0]), dt)
    lib().orc_synth_fbm((I64 * 3)(*dims), params.dtype, C.c_uint32(params.seed), params.octaves,
                        params.base_period, C.c_float(params.threshold), C.c_float(params.vmax),
                        out.ctypes.data_as(C.c_void_p))
    return out


class Swatch(C.Structure):
    _fields_ = [("radial", C.c_int32), ("npoints", C.c_int32), ("nstops", C.c_int32), ("reserved", C.c_int32),
                ("points", C.c_float * 128), ("grad", C.c_float * 4), ("stops", C.c_float * 80)]


def make_swatches(swatches):
    """swatches: list of dicts (radial, points [(x, y)], grad (x0, y0, x1, y1),
    stops [(pos, r, g, b, a)])."""
    arr = (Swatch * max(len(swatches), 1))()
    for k, s in enumerate(swatches):
        arr[k].radial = int(s["radial"])
        arr[k].npoints = len(s["points"])
        arr[k].nstops = len(s["stops"])
        for j, (x, y) in enumerate(s["points"]):
            arr[k].points[2 * j], arr[k].points[2 * j + 1] = x, y
        for j in range(4):
            arr[k].grad[j] = s["grad"][j]
        for j, st in enumerate(s["stops"]):
            for c in range(5):
                arr[k].stops[5 * j + c] = st[c]
    return arr


def raster_tf2d(swatches, tf1d, width, height):
    """CPU restatement of the swatch rasteriser: [height, width, 4] float32,
    row = gradient bin."""
    arr = make_swatches(swatches)
    tf = np.ascontiguousarray(tf1d if tf1d is not None else np.zeros((0, 4)), np.float32)
    out = np.empty((height, width, 4), np.float32)
    lib().orc_raster_tf2d(arr, len(swatches), tf.ctypes.data_as(C.POINTER(C.c_float)), len(tf), width, height,
                          out.ctypes.data_as(C.POINTER(C.c_float)))
    return out
