"""Parameter checks of the seeded synthesis entry points, on the host: a
request whose sizes overflow or exceed the generator's launch limits is
rejected with GBVR_EINVAL before anything reaches the GPU (these run without
one)."""
import ctypes as C

import numpy as np
import pytest

from imagevis3d_gb300 import _lib as L
from imagevis3d_gb300 import synth_params

EINVAL = -1
FAKE_DEV = C.c_void_p(1 << 40)  # never dereferenced: every call below fails its checks first


def _noalloc(p, nbytes=1 << 30):
    return L.lib().gbvr_dev_synth_volume_noalloc(C.byref(p), FAKE_DEV, nbytes, None)


def _alloc(p):
    buf = np.zeros(16, np.uint8)
    return L.lib().gbvr_synth_volume(C.byref(p), buf.ctypes.data_as(C.c_void_p), buf.nbytes)


@pytest.mark.parametrize("dims,dtype", [
    ((1 << 34, 1 << 15, 1 << 15), np.uint16),   # X*Y*Z*2 wraps 64 bits to 0
    ((1 << 40, 1 << 20, 1 << 4), np.uint8),     # X*Y*Z wraps
    (((1 << 62) + 1, 1, 1), np.float32),        # voxel bytes beyond 64 bits
])
def test_wrapping_dims_are_rejected(dims, dtype):
    p = synth_params(dims, dtype, 1, 0, (5.0, 20.0), (0.3, 1.0), 2600.0, vmax=4095.0)
    assert _noalloc(p) == EINVAL
    assert "overflow" in L.last_error() or "dims" in L.last_error()
    assert _alloc(p) == EINVAL


def test_table_size_overflow_is_rejected():
    # nblobs x (1 + X + Y + Z) beyond 2^63 while the voxel count fits
    p = synth_params(((1 << 61), 1, 1), np.uint8, 1, 12000, (5.0, 20.0), (0.3, 1.0), 255.0)
    assert _noalloc(p) == EINVAL
    assert "overflow" in L.last_error()


def test_launch_limits_are_rejected():
    p = synth_params((64, 64, 70000), np.uint8, 1, 1, (5.0, 20.0), (0.3, 1.0), 255.0)
    assert _noalloc(p) == EINVAL and "65535" in L.last_error()
    assert _alloc(p) == EINVAL
    p = synth_params((64, 1 << 31, 1), np.uint8, 1, 1, (5.0, 20.0), (0.3, 1.0), 255.0)
    assert _noalloc(p) == EINVAL and "2^31" in L.last_error()


def test_blob_count_beyond_shared_memory_is_rejected():
    # 13000 blobs fit the no-allocation table array on a 4^3 volume, but the
    # generator keeps a row of blob weights in 48 KiB of shared memory
    p = synth_params((4, 4, 4), np.uint8, 1, 13000, (1.0, 2.0), (0.3, 1.0), 255.0)
    assert _noalloc(p) == EINVAL and "12288" in L.last_error()
    assert _alloc(p) == EINVAL and "12288" in L.last_error()
    p.nblobs = -1
    assert _noalloc(p) == EINVAL


def test_small_output_buffer_is_rejected():
    p = synth_params((64, 64, 64), np.uint8, 1, 4, (5.0, 20.0), (0.3, 1.0), 255.0)
    assert _noalloc(p, nbytes=64 * 64 * 64 - 1) == EINVAL and "too small" in L.last_error()
