"""Python binding of the serving loop (gbvr_server_* in include/gbvr.h)."""
import ctypes as C

import numpy as np

from . import _lib as L
from .renderer import _DT, brick_params


class Server:
    """Datasets + TF presets; requests batched into graph-replayed persistent
    launches, up to `slots` batches in flight on their own streams; with
    device_pool_bytes > 0 the datasets' brick pools share that budget and are
    made resident on demand (least recently used idle ones evicted)."""

    def __init__(self, max_batch=64, fb_budget_bytes=2 << 30, tile_w=8, slots=3, device_pool_bytes=0):
        p = L.ServerParams(max_batch, tile_w, fb_budget_bytes, slots, 0, device_pool_bytes)
        h = C.c_void_p()
        L.call("gbvr_server_create", C.byref(p), C.byref(h))
        self._h = h
        self._bufs = {}

    def close(self):
        if self._h:
            L.lib().gbvr_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def add_volume(self, vol, **bp):
        vol = np.ascontiguousarray(vol)
        dims = (C.c_int64 * 3)(vol.shape[2], vol.shape[1], vol.shape[0])
        i = C.c_int()
        L.call("gbvr_server_add_volume", self._h, vol.ctypes.data_as(C.c_void_p), dims, _DT[vol.dtype],
               C.byref(brick_params(**bp)), C.byref(i))
        return i.value

    def add_synthetic(self, params, **bp):
        i = C.c_int()
        L.call("gbvr_server_add_synthetic", self._h, C.byref(params), C.byref(brick_params(**bp)), C.byref(i))
        return i.value

    def add_tf(self, dataset, mode, tf=None, grad_max=0.0, iso=0.0, iso_rgb=(1, 1, 1), value_range=(0.0, 0.0)):
        i = C.c_int()
        rgb = (C.c_float * 3)(*iso_rgb)
        if tf is None:
            L.call("gbvr_server_add_tf", self._h, dataset, mode, None, 0, 0, grad_max, iso, rgb,
                   value_range[0], value_range[1], C.byref(i))
        else:
            tf = np.ascontiguousarray(tf, np.float32)
            w, h = (tf.shape[0], 1) if tf.ndim == 2 else (tf.shape[1], tf.shape[0])
            L.call("gbvr_server_add_tf", self._h, dataset, mode, tf.ctypes.data_as(L.FP), w, h, grad_max, iso, rgb,
                   value_range[0], value_range[1], C.byref(i))
        return i.value

    def submit(self, dataset, tf, width, height, view, proj, spv=1.0, out=None):
        """Queue a request; its RGBA8 image lands in `out` (a C-contiguous
        (height, width, 4) uint8 array, or a new one) once waited for."""
        if out is None:
            out = np.empty((height, width, 4), np.uint8)
        elif out.shape != (height, width, 4) or out.dtype != np.uint8 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous (height, width, 4) uint8 array")
        r = L.Request()
        r.dataset, r.tf, r.width, r.height = dataset, tf, width, height
        v = np.ascontiguousarray(view, np.float32).ravel()
        p = np.ascontiguousarray(proj, np.float32).ravel()
        for k in range(16):
            r.view[k] = float(v[k])
            r.proj[k] = float(p[k])
        r.samples_per_voxel = spv
        r.out_rgba8 = out.ctypes.data
        t = C.c_uint64()
        L.call("gbvr_server_submit", self._h, C.byref(r), C.byref(t))
        self._bufs[t.value] = out
        return t.value

    def wait(self, ticket, timeout_s=0.0):
        """Pixels and timing of a request.  On a timeout the output buffer stays
        owned here (the server may still write it) and the ticket stays valid."""
        res = L.RequestResult()
        rc = L.lib().gbvr_server_wait(self._h, ticket, timeout_s, C.byref(res))
        if rc == -9:
            raise L.GbvrError(rc, L.last_error())
        out = self._bufs.pop(ticket, None)
        L.check(rc)
        return out, {k: getattr(res, k) for k, _ in L.RequestResult._fields_}

    def stats(self):
        s = L.ServerStats()
        L.call("gbvr_server_get_stats", self._h, C.byref(s))
        return {k: getattr(s, k) for k, _ in L.ServerStats._fields_}

    def autotune(self, width=512, height=512, n=16):
        """Per (voxel type, mode) group: the fastest launch shape on a batch of
        n requests (list of dicts)."""
        out = (L.ServerTune * 12)()
        k = C.c_int()
        L.call("gbvr_server_autotune", self._h, width, height, n, out, 12, C.byref(k))
        return [{f: getattr(out[i], f) for f, _ in L.ServerTune._fields_} for i in range(k.value)]

    def reset_stats(self):
        L.call("gbvr_server_reset_stats", self._h)
