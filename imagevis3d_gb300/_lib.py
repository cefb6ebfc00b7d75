"""ctypes binding of libgbvr.so (the C ABI declared in include/gbvr.h).

The library is loaded from this package directory; there is no fallback: if
the native library is missing or fails to load, every entry point raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbvr.so")

GBVR_OK = 0
GBVR_U8, GBVR_U16, GBVR_F32 = 0, 1, 2
GBVR_CUDA_RAYCASTER = 9
GBVR_RM_1DTRANS, GBVR_RM_2DTRANS, GBVR_RM_ISOSURFACE, GBVR_RM_MIP = 0, 1, 2, 3
GBVR_NEAREST, GBVR_LINEAR = 0, 1
GBVR_SAMPLER_SW, GBVR_SAMPLER_TEX = 0, 1
GBVR_FLAG_FLOAT_FB = 1

ERRORS = {
    -1: "EINVAL", -2: "ECUDA", -3: "ENOMEM", -4: "EIO", -5: "EFORMAT",
    -6: "ECHECKSUM", -7: "ESTATE", -8: "EOVERSIZED", -9: "ETIMEOUT",
}


class BrickParams(C.Structure):
    _fields_ = [("brick_size", C.c_int32), ("overlap", C.c_int32), ("max_lods", C.c_int32),
                ("build_texture", C.c_int32), ("layouts", C.c_int32), ("compression", C.c_int32),
                ("brick_order", C.c_int32), ("reserved", C.c_int32), ("aspect", C.c_double * 3)]


class DatasetInfo(C.Structure):
    _fields_ = [("dims", C.c_int64 * 3), ("dtype", C.c_int32), ("bit_width", C.c_int32),
                ("range", C.c_double * 2), ("lod_count", C.c_int32), ("brick_size", C.c_int32),
                ("overlap", C.c_int32), ("lod_dims", (C.c_int64 * 3) * 16),
                ("lod_bricks", (C.c_int32 * 3) * 16), ("total_bricks", C.c_int64),
                ("device_bytes", C.c_uint64), ("hist1d_size", C.c_int32),
                ("hist2d_max_grad", C.c_float), ("host_bytes", C.c_uint64), ("device_slots", C.c_int32),
                ("compression", C.c_int32), ("host_raw_bytes", C.c_uint64)]


class View(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("proj", C.c_float * 16)]


class Stats(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("samples", C.c_uint64), ("bricks_touched", C.c_uint64),
                ("bricks_skipped", C.c_uint64), ("brick_bytes", C.c_uint64),
                ("brick_misses", C.c_uint64), ("bytes_paged", C.c_uint64), ("h2d_bytes", C.c_uint64),
                ("lod", C.c_int32), ("subframes", C.c_int32), ("gpu_ms", C.c_double),
                ("kernel_ms", C.c_double), ("cells_touched", C.c_uint64), ("cell_bytes", C.c_uint64),
                ("page_ms", C.c_double), ("bytes_paged_compressed", C.c_uint64), ("host_copies", C.c_uint64)]


class TuneResult(C.Structure):
    _fields_ = [("tile_w", C.c_int32), ("ctas_per_sm", C.c_int32), ("candidates", C.c_int32),
                ("best_ms", C.c_float), ("default_ms", C.c_float)]


class BuildStats(C.Structure):
    _fields_ = [("total_ms", C.c_double), ("pyramid_ms", C.c_double), ("cells_ms", C.c_double),
                ("bricks_ms", C.c_double), ("minmax_ms", C.c_double), ("hist1d_ms", C.c_double),
                ("hist2d_ms", C.c_double), ("total_bytes", C.c_uint64), ("pyramid_bytes", C.c_uint64),
                ("cells_bytes", C.c_uint64), ("bricks_bytes", C.c_uint64), ("minmax_bytes", C.c_uint64),
                ("hist1d_bytes", C.c_uint64), ("hist2d_bytes", C.c_uint64), ("level0_bytes", C.c_uint64),
                ("lod_count", C.c_int32), ("layout_copies", C.c_int32)]


class TuneParams(C.Structure):
    _fields_ = [("brick_sizes", C.c_int32 * 4), ("samples_per_step", C.c_int32 * 4)]


class TuneResultEx(C.Structure):
    _fields_ = [("tile_w", C.c_int32), ("ctas_per_sm", C.c_int32), ("brick_size", C.c_int32),
                ("samples_per_step", C.c_int32), ("candidates", C.c_int32), ("best_ms", C.c_float),
                ("default_ms", C.c_float), ("worst_ms", C.c_float)]


class ServerParams(C.Structure):
    _fields_ = [("max_batch", C.c_int32), ("tile_w", C.c_int32), ("fb_budget_bytes", C.c_uint64),
                ("slots", C.c_int32), ("reserved", C.c_int32), ("device_pool_bytes", C.c_uint64)]


class Request(C.Structure):
    _fields_ = [("dataset", C.c_int32), ("tf", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("view", C.c_float * 16), ("proj", C.c_float * 16), ("samples_per_voxel", C.c_float),
                ("reserved", C.c_int32), ("out_rgba8", C.c_void_p)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("batch_size", C.c_int32), ("batch", C.c_uint64),
                ("latency_ms", C.c_double), ("queue_ms", C.c_double), ("gpu_ms", C.c_double)]


class Tf2dSwatch(C.Structure):
    _fields_ = [("radial", C.c_int32), ("npoints", C.c_int32), ("nstops", C.c_int32), ("reserved", C.c_int32),
                ("points", C.c_float * 128), ("grad", C.c_float * 4), ("stops", C.c_float * 80)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("batches", C.c_uint64),
                ("mean_batch", C.c_double), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("max_ms", C.c_double), ("frames_per_s", C.c_double), ("overlap_checked", C.c_uint64),
                ("overlapped", C.c_uint64), ("uploads", C.c_uint64), ("evictions", C.c_uint64),
                ("upload_bytes", C.c_uint64), ("resident_bytes", C.c_uint64)]


class ServerTune(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("mode", C.c_int32), ("tile_w", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("candidates", C.c_int32), ("best_ms", C.c_float), ("default_ms", C.c_float)]


class SynthParams(C.Structure):
    _fields_ = [("dims", C.c_int64 * 3), ("dtype", C.c_int32), ("seed", C.c_uint32),
                ("nblobs", C.c_int32), ("sigma_lo", C.c_float), ("sigma_hi", C.c_float),
                ("amp_lo", C.c_float), ("amp_hi", C.c_float), ("bg_freq", C.c_float),
                ("bg_level", C.c_float), ("bg_amp", C.c_float), ("scale", C.c_float),
                ("noise_kind", C.c_int32), ("noise_amp", C.c_float), ("vmax", C.c_float)]


class FbmParams(C.Structure):
    _fields_ = [("dims", C.c_int64 * 3), ("dtype", C.c_int32), ("seed", C.c_uint32),
                ("octaves", C.c_int32), ("base_period", C.c_int32), ("threshold", C.c_float),
                ("vmax", C.c_float)]


class UvfSummary(C.Structure):
    _fields_ = [("version", C.c_uint64), ("checksum_semantic", C.c_uint64),
                ("checksum", C.c_uint8 * 16), ("checksum_verified", C.c_int32),
                ("nblocks", C.c_int32), ("block_semantics", C.c_uint64 * 32),
                ("dims", C.c_int64 * 3), ("dtype", C.c_int32), ("lod_count", C.c_int32),
                ("brick_size", C.c_int64 * 3), ("overlap", C.c_int64 * 3),
                ("data_offset", C.c_uint64), ("hist1d_size", C.c_int64),
                ("hist2d_nx", C.c_int64), ("hist2d_ny", C.c_int64),
                ("hist2d_max_grad", C.c_float), ("minmax_count", C.c_int64),
                ("minmax_first", C.c_double * 4)]


P = C.c_void_p
I = C.c_int
F = C.c_float
D = C.c_double
SZ = C.c_size_t
I64P = C.POINTER(C.c_int64)
FP = C.POINTER(C.c_float)
U64P = C.POINTER(C.c_uint64)
CP = C.c_char_p

# name -> argument types (every function returns int)
SIGNATURES = {
    "gbvr_last_error": [C.c_char_p, SZ],
    "gbvr_device_info": [C.POINTER(I), C.POINTER(SZ), C.POINTER(SZ)],
    "gbvr_create": [I, C.c_uint32, C.POINTER(P)],
    "gbvr_destroy": [P],
    "gbvr_load_uvf": [P, CP, I, C.POINTER(BrickParams)],
    "gbvr_load_volume": [P, P, I64P, I, C.POINTER(BrickParams)],
    "gbvr_get_dataset_info": [P, C.POINTER(DatasetInfo)],
    "gbvr_get_build_stats": [P, C.POINTER(BuildStats)],
    "gbvr_set_samples_per_step": [P, I],
    "gbvr_autotune_ex": [P, C.POINTER(View), I, C.POINTER(TuneParams), C.POINTER(TuneResultEx)],
    "gbvr_get_hist1d": [P, U64P, SZ],
    "gbvr_get_hist2d": [P, U64P, SZ, SZ, FP],
    "gbvr_get_brick_minmax": [P, I, C.POINTER(D), SZ],
    "gbvr_get_cell_minmax": [P, I, C.POINTER(C.c_float), SZ, C.POINTER(C.c_int32), C.POINTER(C.c_int32)],
    "gbvr_get_brick": [P, I, C.POINTER(C.c_int32), P, SZ, I64P, I64P],
    "gbvr_write_uvf": [P, CP],
    "gbvr_resize": [P, I, I],
    "gbvr_set_render_mode": [P, I],
    "gbvr_set_clip_plane": [P, I, FP],
    "gbvr_set_bboxes": [P, I, I, FP, FP],
    "gbvr_set_iso_relative": [P, F, FP],
    "gbvr_set_blend_precision": [P, I],
    "gbvr_lz4_bound": [SZ],
    "gbvr_lz4_compress": [P, SZ, P, SZ],
    "gbvr_lz4_decompress": [P, SZ, P, SZ],
    "gbvr_zlib_bound": [SZ],
    "gbvr_zlib_compress": [P, SZ, P, SZ],
    "gbvr_zlib_decompress": [P, SZ, P, SZ],
    "gbvr_dev_zlib_decode": [P, P, P, I, P, P],
    "gbvr_dev_lz4_decode": [P, P, P, I, P, P],
    "gbvr_brick_order": [C.POINTER(C.c_int32), C.c_int32, C.c_uint64, C.POINTER(C.c_int32), SZ],
    "gbvr_hilbert3": [C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32],
    "gbvr_set_clearview": [P, I, F, FP, F, F, F, F, F],
    "gbvr_paint_slice": [P, I, C.c_int64, I, I, I],
    "gbvr_paint_path": [P, C.POINTER(View), I, C.POINTER(C.c_int32), U64P, U64P],
    "gbvr_paint_path_capture": [P, C.POINTER(View), I, C.POINTER(C.c_int32), U64P, U64P, P, SZ],
    "gbvr_paint_batch_async": [P, C.POINTER(View), I, I],
    "gbvr_read_framebuffers_async": [P, I, I, I, P, SZ],
    "gbvr_wait_read": [P, I],
    "gbvr_wait_async": [P],
    "gbvr_set_tf1d": [P, FP, I],
    "gbvr_set_tf2d": [P, FP, I, I, F],
    "gbvr_set_value_range": [P, D, D],
    "gbvr_set_iso": [P, F, FP],
    "gbvr_set_lighting": [P, I, FP, FP, FP, FP],
    "gbvr_set_sample_rate": [P, F],
    "gbvr_set_interpolant": [P, I],
    "gbvr_set_sampler": [P, I],
    "gbvr_set_lod_limits": [P, I, I],
    "gbvr_set_view": [P, FP, FP],
    "gbvr_set_background": [P, FP, FP],
    "gbvr_set_early_termination": [P, F],
    "gbvr_set_launch_shape": [P, I, I],
    "gbvr_set_empty_skipping": [P, I],
    "gbvr_autotune": [P, C.POINTER(View), I, C.POINTER(TuneResult)],
    "gbvr_paint": [P],
    "gbvr_paint_batch": [P, C.POINTER(View), I],
    "gbvr_paint_views": [P, C.POINTER(View), I],
    "gbvr_read_framebuffer": [P, I, P, SZ],
    "gbvr_read_framebuffer_f32": [P, I, P, SZ],
    "gbvr_read_framebuffers": [P, I, I, P, SZ],
    "gbvr_capture_single_frame": [P, CP, I],
    "gbvr_capture_view": [P, I, CP, I],
    "gbvr_load_tf1d_file": [CP, I, FP, I, C.POINTER(I)],
    "gbvr_load_tf2d_file": [CP, C.POINTER(I), C.POINTER(I), FP, I, C.POINTER(I), C.POINTER(Tf2dSwatch), I,
                            C.POINTER(I)],
    "gbvr_tf2d_rasterize": [C.POINTER(Tf2dSwatch), I, FP, I, I, I, FP],
    "gbvr_set_tf2d_file": [P, CP, F],
    "gbvr_get_stats": [P, C.POINTER(Stats)],
    "gbvr_set_stats_level": [P, I],
    "gbvr_synth_volume": [C.POINTER(SynthParams), P, SZ],
    "gbvr_load_synthetic": [P, C.POINTER(SynthParams), C.POINTER(BrickParams)],
    "gbvr_load_synthetic_ooc": [P, C.POINTER(SynthParams), C.POINTER(BrickParams), C.c_uint64],
    "gbvr_synth_fbm_volume": [C.POINTER(FbmParams), P, SZ],
    "gbvr_load_synthetic_fbm": [P, C.POINTER(FbmParams), C.POINTER(BrickParams)],
    "gbvr_build_uvf": [P, I64P, I, C.POINTER(BrickParams), CP],
    "gbvr_dev_hist1d": [P, I, C.c_int64, P, I, P],
    "gbvr_dev_hist2d": [P, I, I64P, D, C.c_int64, C.c_int64, P, FP, P],
    "gbvr_dev_downsample": [P, I, I64P, P, P],
    "gbvr_dev_synth_volume_noalloc": [C.POINTER(SynthParams), P, SZ, P],
    "gbvr_orbit_camera": [F, F, F, F, I, I, FP, FP],
    "gbvr_look_at_camera": [FP, FP, FP, F, F, F, I, I, FP, FP],
    "gbvr_server_create": [C.POINTER(ServerParams), C.POINTER(P)],
    "gbvr_server_destroy": [P],
    "gbvr_server_add_volume": [P, P, I64P, I, C.POINTER(BrickParams), C.POINTER(I)],
    "gbvr_server_add_synthetic": [P, C.POINTER(SynthParams), C.POINTER(BrickParams), C.POINTER(I)],
    "gbvr_server_add_tf": [P, I, I, FP, I, I, F, F, FP, D, D, C.POINTER(I)],
    "gbvr_server_submit": [P, C.POINTER(Request), C.POINTER(C.c_uint64)],
    "gbvr_server_wait": [P, C.c_uint64, D, C.POINTER(RequestResult)],
    "gbvr_server_get_stats": [P, C.POINTER(ServerStats)],
    "gbvr_server_reset_stats": [P],
    "gbvr_server_autotune": [P, I, I, I, C.POINTER(ServerTune), I, C.POINTER(I)],
    "gbvr_uvf_inspect": [CP, I, C.POINTER(UvfSummary)],
    "gbvr_uvf_read_volume": [CP, P, SZ],
    "gbvr_uvf_read_hist1d": [CP, U64P, SZ],
    "gbvr_uvf_read_hist2d": [CP, U64P, SZ, FP],
    "gbvr_uvf_write_raster": [CP, CP, P, I64P, I, C.c_int32, C.c_int32, U64P, SZ, U64P, SZ, SZ,
                              F, C.POINTER(D), SZ],
}


class GbvrError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code
        self.msg = msg


_lib = None


# functions that return something other than a status
RESTYPES = {"gbvr_lz4_bound": SZ, "gbvr_lz4_compress": SZ, "gbvr_zlib_bound": SZ, "gbvr_zlib_compress": SZ,
            "gbvr_hilbert3": C.c_uint64}


def lib():
    """Load libgbvr.so once and attach the signatures; raise if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("native library %s is missing: run __graft_entry__.build()" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = RESTYPES.get(name, C.c_int)
    _lib = L
    return L


def last_error():
    buf = C.create_string_buffer(4096)
    lib().gbvr_last_error(buf, 4096)
    return buf.value.decode(errors="replace")


def check(rc):
    if rc != GBVR_OK:
        raise GbvrError(rc, last_error())
    return rc


def call(name, *args):
    return check(getattr(lib(), name)(*args))
