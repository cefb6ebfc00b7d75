"""Host-side mirror of the reference renderer interface, over the C ABI.

Method names follow the Lua methods the reference's scripts call on a
renderer instance (LuaScripts/BatchRenderer.lua:22-41, the RenderWindow
setters of ImageVis3D/UI/RenderWindow.cpp): ``loadDataset``, ``resize``,
``setRenderMode``, ``paint``, ``captureSingleFrame``, ``cleanup`` and so on.
Errors raise ``GbvrError`` carrying the library's status and message.
"""
import ctypes as C

import numpy as np

from . import _lib as L

_DT = {np.dtype(np.uint8): L.GBVR_U8, np.dtype(np.uint16): L.GBVR_U16,
       np.dtype(np.float32): L.GBVR_F32}
_NP = {L.GBVR_U8: np.uint8, L.GBVR_U16: np.uint16, L.GBVR_F32: np.float32}


def _fp(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(L.FP)


def brick_params(brick_size=256, overlap=2, max_lods=0, build_texture=False, layouts=1,
                 aspect=(1, 1, 1), compression=0, brick_order=0):
    """compression: out-of-core host store codec, 0 raw, 1 zlib or 3 (LZ4);
    brick_order: the host store's order of each level's bricks, 0 scanline,
    1 Morton, 2 Hilbert, 3 random."""
    bp = L.BrickParams()
    bp.brick_size = brick_size
    bp.overlap = overlap
    bp.max_lods = max_lods
    bp.build_texture = 1 if build_texture else 0
    bp.layouts = layouts
    bp.compression = compression
    bp.brick_order = brick_order
    for i in range(3):
        bp.aspect[i] = aspect[i]
    return bp


def synth_params(dims, dtype, seed, nblobs, sigma, amp, scale, noise_kind=0, noise_amp=0.0,
                 vmax=255.0, bg_freq=0.0, bg_level=0.0, bg_amp=0.0):
    p = L.SynthParams()
    for i in range(3):
        p.dims[i] = int(dims[i])
    p.dtype = _DT[np.dtype(dtype)]
    p.seed = seed
    p.nblobs = nblobs
    p.sigma_lo, p.sigma_hi = sigma
    p.amp_lo, p.amp_hi = amp
    p.scale = scale
    p.noise_kind = noise_kind
    p.noise_amp = noise_amp
    p.vmax = vmax
    p.bg_freq = bg_freq
    p.bg_level = bg_level
    p.bg_amp = bg_amp
    return p


def fbm_params(dims, dtype, seed, octaves=6, base_period=2, threshold=0.58, vmax=255.0):
    p = L.FbmParams()
    for i in range(3):
        p.dims[i] = int(dims[i])
    p.dtype = _DT[np.dtype(dtype)]
    p.seed = seed
    p.octaves = octaves
    p.base_period = base_period
    p.threshold = threshold
    p.vmax = vmax
    return p


def fbm_volume(params):
    """Generate a seeded fractal volume on the GPU; returns a (z, y, x) array."""
    dims = [params.dims[i] for i in range(3)]
    out = np.empty((dims[2], dims[1], dims[0]), _NP[params.dtype])
    L.call("gbvr_synth_fbm_volume", C.byref(params), out.ctypes.data_as(C.c_void_p), out.nbytes)
    return out


def orbit_camera(azimuth_deg, elevation_deg, radius, fov_deg, width, height):
    """View and projection (row-major float32 4x4) of an orbit camera."""
    v = np.zeros(16, np.float32)
    pr = np.zeros(16, np.float32)
    L.call("gbvr_orbit_camera", azimuth_deg, elevation_deg, radius, fov_deg, width, height,
           v.ctypes.data_as(L.FP), pr.ctypes.data_as(L.FP))
    return v.reshape(4, 4), pr.reshape(4, 4)


def look_at_camera(eye, ref, up, fov_deg, width, height, znear=0.01, zfar=20.0):
    """View and projection of a camera at `eye` looking at `ref`."""
    v = np.zeros(16, np.float32)
    pr = np.zeros(16, np.float32)
    e, c, u = (np.ascontiguousarray(x, np.float32) for x in (eye, ref, up))
    L.call("gbvr_look_at_camera", e.ctypes.data_as(L.FP), c.ctypes.data_as(L.FP), u.ctypes.data_as(L.FP),
           fov_deg, znear, zfar, width, height, v.ctypes.data_as(L.FP), pr.ctypes.data_as(L.FP))
    return v.reshape(4, 4), pr.reshape(4, 4)


def load_tf2d_file(path):
    """Parse a .2dt file: (width, height, 1D TF [n, 4], swatches as a ctypes
    array, swatch count)."""
    w, h, n1, ns = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    L.call("gbvr_load_tf2d_file", path.encode(), C.byref(w), C.byref(h), None, 0, C.byref(n1), None, 0, C.byref(ns))
    tf = np.zeros((max(n1.value, 1), 4), np.float32)
    sw = (L.Tf2dSwatch * max(ns.value, 1))()
    L.call("gbvr_load_tf2d_file", path.encode(), C.byref(w), C.byref(h), tf.ctypes.data_as(L.FP), n1.value,
           C.byref(n1), sw, ns.value, C.byref(ns))
    return w.value, h.value, tf[:n1.value], sw, ns.value


def tf2d_rasterize(swatches, nswatches, tf1d, width, height):
    """GPU rasterisation of swatches over a 1D TF: [height, width, 4] float32,
    row = gradient bin."""
    out = np.empty((height, width, 4), np.float32)
    tf = np.ascontiguousarray(tf1d if tf1d is not None else np.zeros((0, 4)), np.float32)
    L.call("gbvr_tf2d_rasterize", swatches, nswatches, tf.ctypes.data_as(L.FP), len(tf), width, height,
           out.ctypes.data_as(L.FP))
    return out


def synth_volume(params):
    """Generate a seeded volume on the GPU and return it as a (z, y, x) array."""
    dims = [params.dims[i] for i in range(3)]
    out = np.empty((dims[2], dims[1], dims[0]), _NP[params.dtype])
    L.call("gbvr_synth_volume", C.byref(params), out.ctypes.data_as(C.c_void_p), out.nbytes)
    return out


class Renderer:
    """A GBVR_CUDA_RAYCASTER renderer instance (``tuvok.renderer.new``)."""

    def __init__(self, float_fb=False, renderer_type=L.GBVR_CUDA_RAYCASTER):
        h = C.c_void_p()
        L.call("gbvr_create", renderer_type, L.GBVR_FLAG_FLOAT_FB if float_fb else 0, C.byref(h))
        self._h = h
        self.width, self.height = 640, 480
        self._nviews = 1

    # -- lifetime -----------------------------------------------------------
    def cleanup(self):
        if self._h:
            L.lib().gbvr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.cleanup()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.cleanup()

    # -- datasets -----------------------------------------------------------
    def loadDataset(self, path, verify=True, **bp):
        L.call("gbvr_load_uvf", self._h, path.encode(), 1 if verify else 0,
               C.byref(brick_params(**bp)) if bp else None)

    def loadVolume(self, vol, **bp):
        vol = np.ascontiguousarray(vol)
        dims = (C.c_int64 * 3)(vol.shape[2], vol.shape[1], vol.shape[0])
        L.call("gbvr_load_volume", self._h, vol.ctypes.data_as(C.c_void_p), dims, _DT[vol.dtype],
               C.byref(brick_params(**bp)))

    def loadSynthetic(self, params, **bp):
        if isinstance(params, L.FbmParams):
            L.call("gbvr_load_synthetic_fbm", self._h, C.byref(params), C.byref(brick_params(**bp)))
        else:
            L.call("gbvr_load_synthetic", self._h, C.byref(params), C.byref(brick_params(**bp)))

    def loadSyntheticOutOfCore(self, params, device_pool_bytes, **bp):
        L.call("gbvr_load_synthetic_ooc", self._h, C.byref(params), C.byref(brick_params(**bp)), device_pool_bytes)

    def datasetInfo(self):
        info = L.DatasetInfo()
        L.call("gbvr_get_dataset_info", self._h, C.byref(info))
        n = info.lod_count
        return dict(dims=tuple(info.dims), dtype=info.dtype, bit_width=info.bit_width,
                    range=tuple(info.range), lod_count=n, brick_size=info.brick_size,
                    overlap=info.overlap,
                    lod_dims=[tuple(info.lod_dims[i]) for i in range(n)],
                    lod_bricks=[tuple(info.lod_bricks[i]) for i in range(n)],
                    total_bricks=info.total_bricks, device_bytes=info.device_bytes,
                    hist1d_size=info.hist1d_size, hist2d_max_grad=info.hist2d_max_grad,
                    host_bytes=info.host_bytes, device_slots=info.device_slots,
                    compression=info.compression, host_raw_bytes=info.host_raw_bytes)

    def buildStats(self):
        """Device time (ms) and bytes of the last in-core UVF build, per phase."""
        b = L.BuildStats()
        L.call("gbvr_get_build_stats", self._h, C.byref(b))
        return {f: getattr(b, f) for f, _ in L.BuildStats._fields_}

    def getHistogram(self):
        n = self.datasetInfo()["hist1d_size"]
        out = np.zeros(n, np.uint64)
        L.call("gbvr_get_hist1d", self._h, out.ctypes.data_as(L.U64P), n)
        return out

    def get2DHistogram(self):
        nx = self.datasetInfo()["hist1d_size"]
        out = np.zeros((nx, 256), np.uint64)
        mg = C.c_float()
        L.call("gbvr_get_hist2d", self._h, out.ctypes.data_as(L.U64P), nx, 256, C.byref(mg))
        return out, mg.value

    def brickMinMax(self, lod):
        nb = int(np.prod(self.datasetInfo()["lod_bricks"][lod]))
        out = np.zeros((nb, 2), np.float64)
        L.call("gbvr_get_brick_minmax", self._h, lod, out.ctypes.data_as(C.POINTER(C.c_double)), nb)
        return out

    def cellMinMax(self, lod):
        """The level's macro-cell (min, max) grid as a (nz, ny, nx, 2) float32
        array, and the cell edge in voxels."""
        nc = (C.c_int32 * 3)()
        edge = C.c_int32()
        L.call("gbvr_get_cell_minmax", self._h, lod, None, 0, nc, C.byref(edge))
        out = np.zeros((nc[2], nc[1], nc[0], 2), np.float32)
        L.call("gbvr_get_cell_minmax", self._h, lod, out.ctypes.data_as(C.POINTER(C.c_float)), out.size // 2, nc,
               C.byref(edge))
        return out, edge.value

    def getBrick(self, lod, brick):
        b = (C.c_int32 * 3)(*brick)
        o = (C.c_int64 * 3)()
        s = (C.c_int64 * 3)()
        L.call("gbvr_get_brick", self._h, lod, b, None, 0, o, s)
        out = np.empty((s[2], s[1], s[0]), _NP[self.datasetInfo()["dtype"]])
        L.call("gbvr_get_brick", self._h, lod, b, out.ctypes.data_as(C.c_void_p), out.nbytes, o, s)
        return out, tuple(o)

    def writeUVF(self, path):
        L.call("gbvr_write_uvf", self._h, path.encode())

    # -- state --------------------------------------------------------------
    def resize(self, size):
        self.width, self.height = int(size[0]), int(size[1])
        L.call("gbvr_resize", self._h, self.width, self.height)

    def setRenderMode(self, mode):
        L.call("gbvr_set_render_mode", self._h, mode)

    def set1DTrans(self, tf):
        tf, p = _fp(tf)
        L.call("gbvr_set_tf1d", self._h, p, tf.shape[0])

    def set2DTrans(self, tf, max_grad=0.0):
        tf, p = _fp(tf)
        L.call("gbvr_set_tf2d", self._h, p, tf.shape[1], tf.shape[0], max_grad)

    def set2DTransFile(self, path, max_grad=0.0):
        """changed2DTrans from a .2dt file (rasterised on the GPU)."""
        L.call("gbvr_set_tf2d_file", self._h, path.encode(), max_grad)

    def paintPath(self, views, capture=None):
        """Frames of a camera path into framebuffers 0..n-1 (out of core: paging
        of frame i + 1 overlaps the render of frame i).  Returns per-frame
        (lod, misses, bytes_paged) arrays.  capture: a writable buffer of
        n*h*w*4 bytes (page-locked for overlap, e.g. a pinned torch tensor)
        that receives each frame's RGBA8 pixels as soon as the frame is done."""
        arr = self._views(views)
        n = len(views)
        lod = np.zeros(n, np.int32)
        miss = np.zeros(n, np.uint64)
        paged = np.zeros(n, np.uint64)
        args = (self._h, arr, n, lod.ctypes.data_as(C.POINTER(C.c_int32)), miss.ctypes.data_as(L.U64P),
                paged.ctypes.data_as(L.U64P))
        if capture is None:
            L.call("gbvr_paint_path", *args)
        else:
            ptr = capture.data_ptr() if hasattr(capture, "data_ptr") else capture.ctypes.data
            nbytes = capture.numel() * capture.element_size() if hasattr(capture, "numel") else capture.nbytes
            L.call("gbvr_paint_path_capture", *args, C.c_void_p(ptr), nbytes)
        self._nviews = n
        return lod, miss, paged

    def paintSlice(self, axis, index, flip_x=False, flip_y=False, use_mip=False):
        """A 2D render region: the slice `index` (finest-level voxels) across
        `axis` (0 sagittal x, 1 axial y, 2 coronal z), or the maximum along it."""
        L.call("gbvr_paint_slice", self._h, axis, index, int(flip_x), int(flip_y), int(use_mip))
        self._nviews = 1

    def setClipPlane(self, plane, enabled=True):
        """setClipPlane + setClipPlaneEnabled: drop samples with
        a x + b y + c z + d > 0 (world coordinates of the normalised box)."""
        if plane is None:
            L.call("gbvr_set_clip_plane", self._h, 0, None)
            return
        pl, pp = _fp(plane)
        L.call("gbvr_set_clip_plane", self._h, 1 if enabled else 0, pp)

    def setGlobalBBox(self, enabled, rgb=None):
        """setGlobalBBox: draw the dataset box's edges (opaque one-pixel lines
        at their depth)."""
        self._bbox = getattr(self, "_bbox", [False, False])
        self._bbox[0] = bool(enabled)
        keep, gp = _fp(rgb) if rgb is not None else (None, None)
        L.call("gbvr_set_bboxes", self._h, int(self._bbox[0]), int(self._bbox[1]), gp, None)

    def setLocalBBox(self, enabled, rgb=None):
        """setLocalBBox: draw the brick grid of the rendered level."""
        self._bbox = getattr(self, "_bbox", [False, False])
        self._bbox[1] = bool(enabled)
        keep, lp = _fp(rgb) if rgb is not None else (None, None)
        L.call("gbvr_set_bboxes", self._h, int(self._bbox[0]), int(self._bbox[1]), None, lp)

    # ---- ClearView (setCV, setCVIsoValue, setCVColor, setCVSize,
    # setCVContextScale, setCVBorderScale, setCVFocusPos) ----
    def _cv_state(self):
        if not hasattr(self, "_cv"):
            self._cv = dict(on=False, iso=0.0, rgb=(1.0, 1.0, 1.0), size=0.5, context=1.0, border=1.0,
                            fx=-1.0, fy=-1.0)
        return self._cv

    def _cv_apply(self):
        c = self._cv
        keep, rp = _fp(c["rgb"])
        L.call("gbvr_set_clearview", self._h, int(c["on"]), c["iso"], rp, c["size"], c["context"], c["border"],
               c["fx"], c["fy"])

    def _cv_set(self, **kw):
        self._cv_state().update(kw)
        self._cv_apply()

    def setCV(self, enabled):
        self._cv_set(on=bool(enabled))

    def setCVIsoValue(self, value):
        self._cv_set(iso=float(value))

    def setCVColor(self, rgb):
        self._cv_set(rgb=tuple(float(x) for x in rgb))

    def setCVSize(self, size):
        self._cv_set(size=float(size))

    def setCVContextScale(self, scale):
        self._cv_set(context=float(scale))

    def setCVBorderScale(self, scale):
        self._cv_set(border=float(scale))

    def setCVFocusPos(self, x, y):
        """Focus point in pixels (row 0 = top), as the mouse position."""
        self._cv_set(fx=float(x), fy=float(y))

    def setValueRange(self, lo, hi):
        L.call("gbvr_set_value_range", self._h, lo, hi)

    def setIsoValue(self, value, rgb=None):
        c = None
        if rgb is not None:
            arr, c = _fp(rgb)
        L.call("gbvr_set_iso", self._h, value, c)

    def setIsoValueRelative(self, fraction, rgb=None):
        """setIsoValueRelative: the isovalue as a fraction of the value range's top."""
        c = None
        if rgb is not None:
            arr, c = _fp(rgb)
        L.call("gbvr_set_iso_relative", self._h, fraction, c)

    def setBlendPrecision(self, bits):
        """setBlendPrecision (8, 16 or 32): compositing stays FP32."""
        L.call("gbvr_set_blend_precision", self._h, bits)

    def setLightColors(self, ambient, diffuse, specular, direction, enabled=True):
        a, pa = _fp(ambient)
        d, pd = _fp(diffuse)
        s, ps = _fp(specular)
        v, pv = _fp(direction)
        L.call("gbvr_set_lighting", self._h, 1 if enabled else 0, pa, pd, ps, pv)

    def setLightingEnabled(self, enabled):
        L.call("gbvr_set_lighting", self._h, 1 if enabled else 0, None, None, None, None)

    def setSampleRateModifier(self, spv):
        L.call("gbvr_set_sample_rate", self._h, spv)

    def setInterpolant(self, interp):
        L.call("gbvr_set_interpolant", self._h, interp)

    def setSampler(self, sampler):
        L.call("gbvr_set_sampler", self._h, sampler)

    def setLODLimits(self, lo, hi):
        L.call("gbvr_set_lod_limits", self._h, lo, hi)

    def setView(self, view, proj):
        v, pv = _fp(view)
        p, pp = _fp(proj)
        L.call("gbvr_set_view", self._h, pv, pp)

    def setBGColors(self, top, bottom):
        t, pt = _fp(top)
        b, pb = _fp(bottom)
        L.call("gbvr_set_background", self._h, pt, pb)

    def setEarlyTermination(self, alpha):
        L.call("gbvr_set_early_termination", self._h, alpha)

    def setLaunchShape(self, tile_w=8, ctas_per_sm=0):
        L.call("gbvr_set_launch_shape", self._h, tile_w, ctas_per_sm)

    def setEmptySkipping(self, mode):
        L.call("gbvr_set_empty_skipping", self._h, mode)

    def autotune(self, views):
        arr = self._views(views)
        res = L.TuneResult()
        L.call("gbvr_autotune", self._h, arr, len(views), C.byref(res))
        return {k: getattr(res, k) for k, _ in L.TuneResult._fields_}

    def setSamplesPerStep(self, sps):
        L.call("gbvr_set_samples_per_step", self._h, sps)

    def autotuneEx(self, views, brick_sizes=(128, 256, 512), samples_per_step=(1, 2, 4, 8)):
        """Launch shape x brick size x samples per step: the fastest stays set."""
        vs = self._views(views)
        p = L.TuneParams()
        for k, b in enumerate(brick_sizes[:4]):
            p.brick_sizes[k] = b
        for k, v in enumerate(samples_per_step[:4]):
            p.samples_per_step[k] = v
        out = L.TuneResultEx()
        L.call("gbvr_autotune_ex", self._h, vs, len(views), C.byref(p), C.byref(out))
        return {f: getattr(out, f) for f, _ in L.TuneResultEx._fields_}

    # -- paint / readback ---------------------------------------------------
    def paint(self):
        L.call("gbvr_paint", self._h)
        self._nviews = 1

    @staticmethod
    def _views(views):
        arr = (L.View * len(views))()
        for i, (v, p) in enumerate(views):
            v = np.ascontiguousarray(v, np.float32).ravel()
            p = np.ascontiguousarray(p, np.float32).ravel()
            for k in range(16):
                arr[i].view[k] = float(v[k])
                arr[i].proj[k] = float(p[k])
        return arr

    def paintBatch(self, views):
        arr = self._views(views)
        L.call("gbvr_paint_batch", self._h, arr, len(views))
        self._nviews = len(views)

    def paintBatchAsync(self, views, slot):
        """Queue a batch into framebuffer set `slot` (0/1) without waiting."""
        arr = self._views(views)
        L.call("gbvr_paint_batch_async", self._h, arr, len(views), slot)
        self._nviews = len(views)

    def readFramebuffersAsync(self, slot, out, first=0, n=None):
        """Queue the read-back of views [first, first + n) of set `slot` into
        `out` (page-locked memory for an overlap, e.g. a pinned torch tensor)."""
        n = self._nviews - first if n is None else n
        ptr = out.data_ptr() if hasattr(out, "data_ptr") else out.ctypes.data
        nbytes = out.numel() * out.element_size() if hasattr(out, "numel") else out.nbytes
        L.call("gbvr_read_framebuffers_async", self._h, slot, first, n, C.c_void_p(ptr), nbytes)

    def waitRead(self, slot):
        """Wait until the read-backs queued for set `slot` are in host memory."""
        L.call("gbvr_wait_read", self._h, slot)

    def waitAsync(self):
        L.call("gbvr_wait_async", self._h)

    def paintViews(self, views):
        arr = self._views(views)
        L.call("gbvr_paint_views", self._h, arr, len(views))
        self._nviews = len(views)

    def readFramebuffer(self, view=0, as_float=False):
        if as_float:
            out = np.empty((self.height, self.width, 4), np.float32)
            L.call("gbvr_read_framebuffer_f32", self._h, view, out.ctypes.data_as(C.c_void_p), out.nbytes)
        else:
            out = np.empty((self.height, self.width, 4), np.uint8)
            L.call("gbvr_read_framebuffer", self._h, view, out.ctypes.data_as(C.c_void_p), out.nbytes)
        return out

    def readFramebuffers(self, first=0, n=None, out=None):
        """Views [first, first + n) in one copy into `out` (any writable
        buffer of n*h*w*4 bytes, e.g. page-locked memory) or a new array."""
        n = self._nviews - first if n is None else n
        if out is None:
            out = np.empty((n, self.height, self.width, 4), np.uint8)
        ptr = out.data_ptr() if hasattr(out, "data_ptr") else out.ctypes.data
        nbytes = out.numel() * out.element_size() if hasattr(out, "numel") else out.nbytes
        L.call("gbvr_read_framebuffers", self._h, first, n, C.c_void_p(ptr), nbytes)
        return out

    def captureSingleFrame(self, path, preserve_transparency=True):
        L.call("gbvr_capture_single_frame", self._h, path.encode(), 1 if preserve_transparency else 0)

    def setStatsLevel(self, level):
        L.call("gbvr_set_stats_level", self._h, level)

    def stats(self):
        s = L.Stats()
        L.call("gbvr_get_stats", self._h, C.byref(s))
        return {k: getattr(s, k) for k, _ in L.Stats._fields_}
