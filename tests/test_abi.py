"""The C-ABI library loads and exports every function include/gbvr.h declares
(no compute calls: this runs without a GPU)."""
import ctypes as C
import os
import re

import numpy as np

from imagevis3d_gb300 import _lib as L
from tests.conftest import ROOT


def declared_functions():
    text = open(os.path.join(ROOT, "include", "gbvr.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|size_t|uint64_t)\s+(gbvr_\w+)\s*\(", text, flags=re.M)))


def test_every_declared_symbol_is_exported_and_bound():
    names = declared_functions()
    assert len(names) >= 40
    lib = L.lib()
    for n in names:
        assert hasattr(lib, n), n
        assert n in L.SIGNATURES, "binding lacks %s" % n
    assert sorted(L.SIGNATURES) == names


def test_struct_layouts_match_the_c_compiler(tmp_path):
    """The ctypes mirrors of the header's POD structs have the C compiler's
    sizes and field offsets."""
    import shutil
    import subprocess
    import pytest
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    structs = {"gbvr_brick_params": L.BrickParams, "gbvr_dataset_info": L.DatasetInfo,
               "gbvr_view": L.View, "gbvr_stats": L.Stats, "gbvr_synth_params": L.SynthParams,
               "gbvr_uvf_summary": L.UvfSummary, "gbvr_fbm_params": L.FbmParams,
               "gbvr_tune_result": L.TuneResult, "gbvr_server_params": L.ServerParams,
               "gbvr_request": L.Request, "gbvr_request_result": L.RequestResult,
               "gbvr_server_stats": L.ServerStats, "gbvr_tf2d_swatch": L.Tf2dSwatch}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gbvr.h"', "int main(void){"]
    for cname, py in structs.items():
        lines.append('printf("%%zu\\n", sizeof(%s));' % cname)
        for f, _ in py._fields_:
            lines.append('printf("%%zu\\n", offsetof(%s, %s));' % (cname, f))
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    want = []
    for cname, py in structs.items():
        want.append(C.sizeof(py))
        want.extend(getattr(py, f).offset for f, _ in py._fields_)
    assert got == want


def test_errors_without_gpu_are_statuses():
    h = C.c_void_p()
    rc = L.lib().gbvr_create(1, 0, C.byref(h))  # an OpenGL type: not this library's
    assert rc == -1 and "GBVR_CUDA_RAYCASTER" in L.last_error()
    rc = L.lib().gbvr_paint(None)
    assert rc == -1


def test_renderer_calls_reject_a_null_handle():
    """Every renderer call checks its handle before anything else: a null
    renderer is GBVR_EINVAL with a message, and no CUDA call is made."""
    lib = L.lib()
    rgb = (C.c_float * 3)(1.0, 0.5, 0.25)
    plane = (C.c_float * 4)(1.0, 0.0, 0.0, 0.0)
    calls = [
        ("gbvr_set_render_mode", (None, 0)),
        ("gbvr_set_iso", (None, C.c_float(0.5), rgb)),
        ("gbvr_set_iso_relative", (None, C.c_float(0.5), rgb)),
        ("gbvr_set_blend_precision", (None, 32)),
        ("gbvr_set_sample_rate", (None, C.c_float(1.0))),
        ("gbvr_set_interpolant", (None, 1)),
        ("gbvr_set_lod_limits", (None, 0, 4)),
        ("gbvr_set_background", (None, rgb, rgb)),
        ("gbvr_set_empty_skipping", (None, 2)),
        ("gbvr_set_clip_plane", (None, 1, plane)),
        ("gbvr_set_bboxes", (None, 1, 1, rgb, rgb)),
        ("gbvr_set_clearview", (None, 1, C.c_float(0.5), rgb, C.c_float(0.5), C.c_float(1.0), C.c_float(1.0),
                                C.c_float(0.0), C.c_float(0.0))),
        ("gbvr_wait_read", (None, 0)),
        ("gbvr_paint", (None,)),
    ]
    for name, args in calls:
        rc = getattr(lib, name)(*args)
        assert rc == -1, name
        assert "null renderer" in L.last_error(), name


def test_orbit_camera_is_host_math():
    v = np.zeros(16, np.float32)
    p = np.zeros(16, np.float32)
    L.call("gbvr_orbit_camera", 90.0, 0.0, 4.0, 45.0, 640, 480, v.ctypes.data_as(L.FP),
           p.ctypes.data_as(L.FP))
    V = v.reshape(4, 4).astype(np.float64)
    eye = -np.linalg.inv(V[:3, :3]) @ V[:3, 3]
    assert np.allclose(eye, [4, 0, 0], atol=1e-5)
    P = p.reshape(4, 4)
    assert abs(P[1, 1] - 1 / np.tan(np.radians(22.5))) < 1e-5
    assert abs(P[0, 0] * 640 / 480 - P[1, 1]) < 1e-5
