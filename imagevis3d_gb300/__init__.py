"""GB300-native bricked volume raycaster and UVF build (ImageVis3D hot path).

The product is the native library ``libgbvr.so`` (C ABI in include/gbvr.h);
this package is its Python binding.  Nothing here computes on the CPU: when the
library is missing the binding raises instead of falling back.
"""
from ._lib import (GbvrError, GBVR_U8, GBVR_U16, GBVR_F32, GBVR_CUDA_RAYCASTER,  # noqa: F401
                   GBVR_RM_1DTRANS, GBVR_RM_2DTRANS, GBVR_RM_ISOSURFACE, GBVR_RM_MIP, GBVR_NEAREST,
                   GBVR_LINEAR, GBVR_SAMPLER_SW, GBVR_SAMPLER_TEX, lib)
from .renderer import (Renderer, brick_params, fbm_params, fbm_volume, load_tf2d_file, look_at_camera,  # noqa: F401
                       orbit_camera, synth_params, synth_volume, tf2d_rasterize)
from .server import Server  # noqa: F401
from . import workloads  # noqa: F401
