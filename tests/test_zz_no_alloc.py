"""gbvr_dev_synth_volume_noalloc: seeded synthesis into a caller-owned device
buffer with no device allocation (its generator tables live in a fixed
device array inside the library).  It must produce exactly the volume of the
allocating entry point gbvr_synth_volume, call after call, since every call
reuses the same array.  This file is collected last so that a run stopping at
the first failure has run every other test before it."""
import ctypes as C

import numpy as np
import pytest

from imagevis3d_gb300 import _lib as L
from imagevis3d_gb300 import synth_params, synth_volume, workloads

pytestmark = pytest.mark.gpu


def _noalloc(params, torch):
    dims = [params.dims[i] for i in range(3)]
    dt = {L.GBVR_U8: torch.uint8, L.GBVR_U16: torch.int16, L.GBVR_F32: torch.float32}[params.dtype]
    # the caller owns the output buffer (allocated here, by the test)
    out = torch.empty((dims[2], dims[1], dims[0]), dtype=dt, device="cuda")
    L.call("gbvr_dev_synth_volume_noalloc", C.byref(params), C.c_void_p(out.data_ptr()),
           out.numel() * out.element_size(), None)
    return out


def _host(out, params):
    npdt = {L.GBVR_U8: np.uint8, L.GBVR_U16: np.uint16, L.GBVR_F32: np.float32}[params.dtype]
    return out.cpu().numpy().view(npdt)


def test_noalloc_matches_allocating_entry_point_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    a = workloads.config1().synth                                   # 128^3 uint8, uniform noise
    b = synth_params((96, 80, 72), np.uint16, 77, 16, (5.0, 20.0), (0.3, 1.0), 2600.0,
                     noise_kind=2, noise_amp=20.0, vmax=4095.0, bg_freq=1.0, bg_level=0.15,
                     bg_amp=0.1)                                     # u16, background + Gaussian
    ga = _noalloc(a, torch)
    gb = _noalloc(b, torch)  # same stream, right after: reuses the table array
    torch.cuda.synchronize()
    # bit-exact, the tolerance of every synthesis test
    assert np.array_equal(_host(ga, a), synth_volume(a))
    assert np.array_equal(_host(gb, b), synth_volume(b))
    # and again in the other order: nothing of the previous call leaks in
    ga2 = _noalloc(a, torch)
    torch.cuda.synchronize()
    assert np.array_equal(_host(ga2, a), synth_volume(a))


def test_noalloc_allocates_no_device_memory():
    """The defining property: after the first call on the device (its set-up),
    further calls leave the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    a = workloads.config1().synth
    b = synth_params((96, 80, 72), np.uint16, 77, 16, (5.0, 20.0), (0.3, 1.0), 2600.0, noise_kind=2,
                     noise_amp=20.0, vmax=4095.0, bg_freq=1.0, bg_level=0.15, bg_amp=0.1)
    outs = []
    for p in (a, b):  # outputs owned by the caller, allocated before measuring
        dims = [p.dims[i] for i in range(3)]
        dt = torch.uint8 if p.dtype == L.GBVR_U8 else torch.int16
        outs.append(torch.empty((dims[2], dims[1], dims[0]), dtype=dt, device="cuda"))

    def call(p, out):
        L.call("gbvr_dev_synth_volume_noalloc", C.byref(p), C.c_void_p(out.data_ptr()),
               out.numel() * out.element_size(), None)

    call(a, outs[0])  # warm-up: set-up on this device, kernel loaded
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        call(a, outs[0])
        call(b, outs[1])
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert np.array_equal(_host(outs[1], b), synth_volume(b))


@pytest.mark.filterwarnings("ignore:The CUDA Graph is empty")
def test_noalloc_is_refused_during_stream_capture():
    """A captured call would read the shared host tables at replay time; it
    is refused, and nothing is queued into the capture."""
    torch = pytest.importorskip("torch")
    a = workloads.config1().synth
    out = torch.empty((128, 128, 128), dtype=torch.uint8, device="cuda")
    _noalloc(a, torch)  # set-up before any capture
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            rc = L.lib().gbvr_dev_synth_volume_noalloc(C.byref(a), C.c_void_p(out.data_ptr()),
                                                       out.numel(), C.c_void_p(s.cuda_stream))
    assert rc == -1 and "captured" in L.last_error()


def test_noalloc_rejects_tables_beyond_its_capacity():
    torch = pytest.importorskip("torch")
    big = synth_params((1024, 1024, 1024), np.uint16, 1, 200, (5.0, 20.0), (0.3, 1.0), 2600.0,
                       vmax=4095.0)
    buf = torch.empty(16, dtype=torch.uint8, device="cuda")
    rc = L.lib().gbvr_dev_synth_volume_noalloc(C.byref(big), C.c_void_p(buf.data_ptr()), 16, None)
    assert rc == -1
    msg = L.last_error()
    assert "262144" in msg and "no-allocation" in msg
