"""Shared helpers of the GPU parity tests: image error against the FP64
oracle, with the tolerance of the raycaster's accuracy contract."""
import numpy as np

# Per-channel tolerance of the FP32 GPU image against the FP64 oracle image
# (RGBA in [0, 1]): max |error| <= 2/255 and RMS <= 0.5/255.
TOL_MAX = 2.0 / 255.0
TOL_RMS = 0.5 / 255.0


def image_error(gpu, ref):
    """Max and RMS per-channel error of the images: both saturated to [0, 1]
    first, as the RGBA8 framebuffer stores them (lit colours can exceed 1 in
    the float framebuffer, e.g. on specular highlights)."""
    g = np.clip(np.asarray(gpu, np.float64), 0.0, 1.0)
    r = np.clip(np.asarray(ref, np.float64), 0.0, 1.0)
    d = np.abs(g - r)
    return float(d.max()), float(np.sqrt(np.mean(d * d)))


def assert_close(gpu, ref, tol_max=TOL_MAX, tol_rms=TOL_RMS):
    mx, rms = image_error(gpu, ref)
    assert mx <= tol_max and rms <= tol_rms, "max %.5f (tol %.5f) rms %.6f (tol %.6f)" % (mx, tol_max, rms, tol_rms)
    return mx, rms
