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


def perturbed_view(view, eps, rng):
    """The view matrix with each entry scaled by (1 + eps * N(0, 1)): a camera
    that differs from `view` by rounding-sized amounts (FP32's unit roundoff is
    6e-8) in every entry, as the kernel's single-precision ray setup does."""
    v = np.asarray(view, np.float64)
    return (v * (1.0 + eps * rng.standard_normal(v.shape))).astype(np.float32)


def backward_error(gpu, ref, oracle, view, tol_max=TOL_MAX, eps=(3e-7, 1e-6, 2e-6), tries=48, seed=0):
    """Image error where the image is ill-conditioned at a few pixels (an
    isosurface of a fractal: a ray grazing the surface hits on one side of a
    sample or the next depending on the 7th digit of its position).  A pixel
    within tol_max of the FP64 oracle is matched; each other pixel is matched
    when the FP64 oracle at some camera perturbed by at most max(eps) relative
    per view-matrix entry reproduces it within tol_max (backward error: the GPU
    pixel is the exact pixel of a camera within FP32 rounding of the given
    one; 2e-6 is about 16 units in the last place of FP32, the scale of the
    kernel's single-precision ray setup from a camera thousands of voxels
    away).  oracle(view, idx) renders the pixels ref[idx] (RGBA [m, 4]) at a
    camera.  Returns max / RMS of the forward error, the pixels beyond tol_max
    forward, the max / RMS (per channel) against each pixel's best match, and
    the pixels no perturbed camera reproduced."""
    g = np.clip(np.asarray(gpu, np.float64), 0.0, 1.0)
    r = np.clip(np.asarray(ref, np.float64), 0.0, 1.0)
    dif = np.abs(g - r)          # each pixel's channel errors against its best match so far
    fwd_max, fwd_rms = float(dif.max(initial=0.0)), float(np.sqrt(np.mean(dif ** 2))) if dif.size else 0.0
    best = dif.max(axis=1)
    bad = np.flatnonzero(best > tol_max)
    rng = np.random.default_rng(seed)
    left = bad
    for t in range(tries):
        if left.size == 0:
            break
        out = np.clip(np.asarray(oracle(perturbed_view(view, eps[t % len(eps)], rng), left), np.float64), 0.0, 1.0)
        d = np.abs(g[left] - out)
        better = d.max(axis=1) < best[left]
        dif[left[better]] = d[better]
        best[left[better]] = d[better].max(axis=1)
        left = left[best[left] > tol_max]
    return {"max": fwd_max, "rms": fwd_rms, "pixels": int(len(g)), "beyond_tol": int(bad.size),
            "backward_max": float(best.max(initial=0.0)),
            "backward_rms": float(np.sqrt(np.mean(dif ** 2))) if dif.size else 0.0,
            "unresolved": left.tolist(), "unresolved_err": np.round(best[left], 4).tolist()}


def assert_close_backward(gpu, ref, oracle, view, tol_max=TOL_MAX, tol_rms=TOL_RMS, max_frac=0.02, **kw):
    """backward_error within tolerance: every pixel matched within tol_max
    (forward, or by a perturbed camera), at most max_frac of them only by a
    perturbed camera, and the RMS against the best matches within tol_rms."""
    e = backward_error(gpu, ref, oracle, view, tol_max=tol_max, **kw)
    assert e["beyond_tol"] <= max_frac * max(e["pixels"], 1), "%d of %d pixels beyond tolerance (max %.4f)" % (
        e["beyond_tol"], e["pixels"], e["max"])
    assert not e["unresolved"], "pixels %s not reproduced by any perturbed camera (best %s)" % (
        e["unresolved"], e["unresolved_err"])
    assert e["backward_rms"] <= tol_rms, "rms %.6f (tol %.6f)" % (e["backward_rms"], tol_rms)
    return e
