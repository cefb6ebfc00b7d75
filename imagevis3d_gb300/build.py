"""Build recipe for the native library (libgbvr.so) and the headless driver.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); host C++ units with g++.  Units
compile in parallel; the CUDA runtime is linked statically so the library has
no path dependency on libcudart.  Outputs stay in-tree beside this file.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbvr.so")
DRIVER = os.path.join(HERE, "gbvr_batch")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

CUDA_UNITS = ["kernels_render.cu", "kernels_build.cu", "gbvr_api.cu", "noalloc.cu", "tf2d.cu"]
HOST_UNITS = ["uvf.cpp", "uvf_api.cpp", "image_io.cpp", "lz4.cpp", "deflate.cpp", "brick_order.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p.stderr


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".h")]
    headers.append(os.path.join(INCLUDE, "gbvr.h"))
    jobs = []
    objs = []
    for u in CUDA_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OBJ, u + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            # host code: one rounding per operation (no FMA contraction on
            # any host CPU), so host-side FP64 geometry is reproducible
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v", "-c", src, "-o", obj])
    for u in HOST_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OBJ, u + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", src, "-o", obj])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            logs = list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lpthread", "-ldl", "-lrt"])
        os.replace(LIB + ".tmp", LIB)
    drv_src = os.path.join(CSRC, "gbvr_batch.cpp")
    if os.path.exists(drv_src) and (force or _stale(DRIVER, [drv_src, LIB])):
        _run(["g++", "-O2", "-std=c++17", drv_src, "-o", DRIVER, "-L" + HERE, "-lgbvr",
              "-Wl,-rpath,$ORIGIN"])
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
