"""Benchmark: batched persistent raycast of the 1024^3 uint16 bricked volume.

Workload (one step): a 64-view orbit at 1920x1080 of a 1024^3 uint16 volume
with 12-bit values (64 seeded blobs on a low-frequency background + Gaussian
noise), bricked as 256^3 bricks with 2 ghost voxels (125 bricks at LOD 0,
4 LOD levels), 4096-entry 1D TF, 1.5 samples per voxel, finest level, one
persistent launch over all 64 views.  Inputs are seeded synthetic data; no
dataset ships with the reference for this size.

Printed line (one JSON object, rank 0):
  value     frames/s of the batched persistent kernel, device time (CUDA
            events on the launching stream), volume resident in HBM.  The
            brick pool (2.3 GB) is larger than L2, so no flush is needed.
  e2e       frames/s through the public API with host buffers: paint_batch
            (view descriptors host->device) + read back of all 64 RGBA8
            framebuffers into host memory, wall clock.
  roofline  dominant kernel (the persistent raycast): algorithmic bytes per
            launch = stored bytes of the distinct non-skipped bricks each view
            samples, summed over views, / kernel time, against the measured
            HBM copy bandwidth.
  cpu_baseline  the FP64 CPU oracle (a port: the reference's raycaster is
            GLSL in an absent submodule) on a bounded pixel sample of view 0.

--impl reference times that CPU implementation alone (all host threads) on
the same workload and metric.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/s & Gsamples/s, batched vs per-view, <=2/255 vs FP64 oracle; p99 ms"


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        """Start sampling every 50 ms; returns once the first sample is in, so
        the samples that follow fall inside the timed region.  The first one
        (taken before the region) is dropped."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.first = threading.Event()
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self.first.wait(timeout=5.0)
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            if self.first.is_set():
                self.lines.append(line.strip())
            self.first.set()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(wl, vol, view, proj, seconds, threads, rng_seed):
    """Oracle render of seeded pixel batches of one view until `seconds` of
    CPU work; returns (pixels/s, samples/s, pixels, the oracle rgba, pixel ids)."""
    import numpy as np
    from oracle import orc
    rng = np.random.default_rng(rng_seed)
    npix_total = wl.width * wl.height
    done, ns, t0 = 0, 0, time.perf_counter()
    pix_all, ref_all = [], []
    batch = 2048
    while True:
        pix = rng.integers(0, npix_total, batch)
        ref, n = orc.render(vol, view, proj, wl.width, wl.height, wl.tf, spv=wl.spv,
                            value_range=wl.value_range, pixels=pix, threads=threads)
        done += batch
        ns += n
        pix_all.append(pix)
        ref_all.append(ref)
        el = time.perf_counter() - t0
        if el >= seconds:
            break
        batch = min(batch * 2, 65536)
    return done / el, ns / el, done, np.concatenate(ref_all), np.concatenate(pix_all), el


def run_reference(args):
    """The reference's CPU implementation of the path (the FP64 oracle port:
    Tuvok's raycaster is unbuildable here), all host threads, per step a
    bounded pixel sample of view 0 of the same workload.  Nothing of the GPU
    library is imported or loaded on this arm: the scene (volume parameters,
    TF, cameras) comes from oracle.scenes, the cameras from the oracle's own
    FP64 camera code."""
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    from oracle import orc, scenes
    wl = scenes.config2(size=args.size, nviews=64)
    vol = orc.synth_blobs(wl.synth)
    threads = orc.max_threads()
    view, proj = wl.views[0]
    for _ in range(args.warmup):
        cpu_sample(wl, vol, view, proj, 0.5, threads, 1)
    rates, srates, total_t = [], [], 0.0
    # per step a sample of ref_seconds of CPU work, shortened so that the
    # whole run stays near two minutes
    per = min(args.ref_seconds, max(1.0, 120.0 / max(args.steps, 1)))
    for s in range(args.steps):
        pr, sr, n, _, _, el = cpu_sample(wl, vol, view, proj, per, threads, 100 + s)
        rates.append(pr / (wl.width * wl.height))
        srates.append(sr)
        total_t += el
    fps = statistics.mean(rates)
    out = {
        "metric": METRIC, "value": fps, "unit": "frames/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * total_t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded)",
        "config": {"workload": wl.name, "views": 64, "width": wl.width, "height": wl.height,
                   "samples_per_voxel": wl.spv},
        "gsamples_per_s": statistics.mean(srates) / 1e9,
        "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": "seeded pixel subsets of view 0, %.1f s of CPU work per step, "
                                   "frames/s = pixels/s / (%d*%d)" % (per, wl.width, wl.height)},
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    return 0


PROFILE_CSV = os.path.join(ROOT, "profiles", "raycast_persistent_1024cube_u16_8views.ncu.csv")


def profile_counters():
    """Counters of one ncu capture of the persistent raycast kernel on the
    8-view case of this workload (profiles/*.ncu.csv: the raw page of the
    capture, base units, reduced to the columns used here).  None when the
    file is absent.  The bench scales them to its own launch by ratios it
    measures itself (algorithmic bytes and samples of the same 8 views)."""
    import csv
    try:
        rows = list(csv.reader(open(PROFILE_CSV)))
    except OSError:
        return None
    hdr, vals = rows[0], rows[-1]
    out = {}
    for k, v in zip(hdr, vals):
        try:
            out[k] = float(v.replace(",", ""))
        except ValueError:
            out[k] = v
    return out


def run_c3(args):
    """Sparse fractal workload: 2048^3 uint8 fBm, 2D TF +
    Phong DVR and isosurfaces at 2560x1440, plus the GPU 2D histogram of the
    8 GiB level.  Prints one JSON line of its own."""
    import numpy as np
    import torch
    from imagevis3d_gb300 import (GBVR_RM_2DTRANS, GBVR_RM_ISOSURFACE, Renderer, workloads)
    from imagevis3d_gb300 import _lib as L
    import ctypes as C
    wl = workloads.config3(size=args.size if args.size != 1024 else 2048, nviews=args.views if args.views != 64 else 16)
    r = Renderer()
    t0 = time.perf_counter()
    # both blocked copies: the isosurfaces sample the overlapped blocks, the
    # 2D-TF DVR the compact ones
    r.loadSynthetic(wl.synth, **wl.brick, layouts=6)
    build_s = time.perf_counter() - t0
    info = r.datasetInfo()
    r.resize((wl.width, wl.height))
    r.setRenderMode(GBVR_RM_2DTRANS)
    r.set2DTrans(wl.tf, info["hist2d_max_grad"] * 0.5)
    r.setValueRange(*wl.value_range)
    r.setSampleRateModifier(wl.spv)
    tune = r.autotune(wl.views)
    for _ in range(args.warmup):
        r.paintBatch(wl.views)
    ms = []
    for _ in range(args.steps):
        r.paintBatch(wl.views)
        ms.append(r.stats()["kernel_ms"])
    st = r.stats()
    dvr_fps = len(wl.views) * args.steps / (sum(ms) / 1000.0)
    r.paintViews(wl.views)
    pms = []
    for _ in range(args.steps):
        r.paintViews(wl.views)
        pms.append(r.stats()["gpu_ms"])
    dvr_plain = len(wl.views) * args.steps / (sum(pms) / 1000.0)
    # error against the FP64 oracle (voxels evaluated on demand from the
    # fractal's rule): seeded pixel subsets of one view's RGBA8 frame, so the
    # 8-bit rounding is included
    from oracle import orc
    proc = orc.ProceduralFbm(wl.synth)
    erng = np.random.default_rng(workloads.SEED + 33)
    errs = {}

    def frame_error(key, view_idx, kw, covered_thr):
        img = r.readFramebuffer(view_idx).reshape(-1, 4).astype(np.float64) / 255.0
        cov = np.flatnonzero(img[:, 3] > covered_thr)
        ncov = 800 if kw.get("mode") == 2 else 200
        pix = np.concatenate([erng.choice(cov, min(ncov, cov.size), replace=False) if cov.size else
                              np.zeros(0, np.int64), erng.integers(0, img.shape[0], 60)])
        v, p = wl.views[view_idx]
        ref, _ = orc.render(proc, v, p, wl.width, wl.height, wl.tf, value_range=wl.value_range, pixels=pix,
                            threads=orc.max_threads(), **kw)
        g = np.clip(img[pix], 0, 1)
        rr = np.clip(ref, 0, 1)
        if kw.get("mode") == 2:
            # silhouette rays may hit on one side only; where both hit, a pixel
            # beyond tolerance is matched against the oracle at cameras
            # perturbed by FP32-rounding-sized amounts (the isosurface of the
            # fractal is ill-conditioned at a few pixels)
            same = np.flatnonzero((g[:, 3] > 0.5) == (rr[:, 3] > 0.5))
            errs[key + "_hit_mismatch"] = float(1.0 - same.size / len(g))
            from tests.gpu_util import backward_error

            def oracle(view, sub):
                return orc.render(proc, view, p, wl.width, wl.height, wl.tf, value_range=wl.value_range,
                                  pixels=pix[same[sub]], threads=orc.max_threads(), **kw)[0]

            e = backward_error(g[same], rr[same], oracle, v)
            errs[key] = {k: e[k] for k in ("max", "rms", "pixels", "beyond_tol", "backward_max", "backward_rms")}
            errs[key]["unresolved"] = len(e["unresolved"])
            return
        d = np.abs(g - rr)
        errs[key] = {"max": float(d.max()), "rms": float(np.sqrt((d * d).mean())), "pixels": int(len(g))}

    r.paintBatch(wl.views)
    frame_error("dvr_2dtf_phong", 0, dict(mode=1, grad_max=info["hist2d_max_grad"] * 0.5), 0.02)
    r.setRenderMode(GBVR_RM_ISOSURFACE)
    iso_fps = []
    for ii, iso in enumerate(wl.isovalues):
        r.setIsoValue(iso, (0.8, 0.8, 0.9))
        r.paintBatch(wl.views)
        ims = []
        for _ in range(args.steps):
            r.paintBatch(wl.views)
            ims.append(r.stats()["kernel_ms"])
        iso_fps.append(len(wl.views) * args.steps / (sum(ims) / 1000.0))
        frame_error("iso_%d" % ii, 3, dict(mode=2, iso=iso, iso_rgb=(0.8, 0.8, 0.9)), 0.5)
    errs["tol_max"], errs["tol_rms"] = 2 / 255, 0.5 / 255
    errs["note"] = ("RGBA8 frames (8-bit rounding included) vs the FP64 oracle, seeded pixel subsets; iso_*: "
                    "max/rms forward, beyond_tol pixels, backward_max/rms against the oracle at cameras perturbed "
                    "by <= 2e-6 relative per view-matrix entry")
    r.cleanup()
    # GPU 2D histogram of the 8 GiB level, device resident
    n = wl.synth.dims[0] * wl.synth.dims[1] * wl.synth.dims[2]
    vol = torch.empty(n, dtype=torch.uint8, device="cuda")
    hist = torch.zeros(256 * 256, dtype=torch.int64, device="cuda")
    # regenerate the level into the device buffer through a renderer-free path
    from imagevis3d_gb300 import fbm_volume
    host = fbm_volume(wl.synth)
    vol.copy_(torch.from_numpy(host.reshape(-1)))
    dims = (C.c_int64 * 3)(*[wl.synth.dims[i] for i in range(3)])
    mg = C.c_float()
    stream = torch.cuda.current_stream().cuda_stream
    L.call("gbvr_dev_hist2d", C.c_void_p(vol.data_ptr()), 0, dims, 255.0, 256, 1, C.c_void_p(hist.data_ptr()),
           C.byref(mg), C.c_void_p(stream))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    hms = []
    for _ in range(3):
        hist.zero_()
        e0.record()
        L.call("gbvr_dev_hist2d", C.c_void_p(vol.data_ptr()), 0, dims, 255.0, 256, 1, C.c_void_p(hist.data_ptr()),
               C.byref(mg), C.c_void_p(stream))
        e1.record()
        torch.cuda.synchronize()
        hms.append(e0.elapsed_time(e1))
    hist_ms = min(hms)
    pk = peaks()
    out = {
        "metric": "frames/s (2D TF + Phong DVR, batched) & isosurface frames/s & 2D histogram GB/s",
        "value": dvr_fps, "unit": "frames/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sum(ms) / len(ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic (seeded fBm volume)",
        "config": {"workload": wl.name, "volume": "%d^3 uint8" % wl.synth.dims[0], "views": len(wl.views),
                   "brick_layouts": "x-fastest + 4^3 blocks (2D TF) + overlapped 5^3 blocks (isosurfaces)",
                   "width": wl.width, "height": wl.height, "tf": "2D 256x256, 3 Gaussian-ellipse widgets, Phong",
                   "bricks_empty_fraction": None},
        "per_view_plain_fps": dvr_plain, "batched_vs_per_view": dvr_fps / dvr_plain,
        "isosurface_fps": dict(zip(["%.1f" % v for v in wl.isovalues], iso_fps)),
        "gsamples_per_s": st["samples"] / (ms[-1] / 1000.0) / 1e9,
        "uvf_build_s": build_s,
        "image_error_vs_fp64": errs,
        "hist2d": {"ms": hist_ms, "gbps_read_3_passes": 3 * n / (hist_ms / 1000.0) / 1e9,
                   "peak_gbps": pk["hbm_gbs"] if pk else None},
        "autotune": tune,
    }
    print(json.dumps(out))
    return 0


def level_from_bricks(r, lod):
    """The flat level `lod` of a loaded dataset, assembled from its bricks'
    interiors (host copies; out-of-core bricks come from the host store)."""
    import numpy as np
    info = r.datasetInfo()
    X, Y, Z = info["lod_dims"][lod]
    nb = info["lod_bricks"][lod]
    g = info["overlap"]
    interior = info["brick_size"] - 2 * g
    out = None
    for bz in range(nb[2]):
        for by in range(nb[1]):
            for bx in range(nb[0]):
                v, o = r.getBrick(lod, (bx, by, bz))
                if out is None:
                    out = np.empty((Z, Y, X), v.dtype)
                x0, y0, z0 = bx * interior, by * interior, bz * interior
                x1, y1, z1 = min(x0 + interior, X), min(y0 + interior, Y), min(z0 + interior, Z)
                out[z0:z1, y0:y1, x0:x1] = v[g:g + z1 - z0, g:g + y1 - y0, g:g + x1 - x0]
    return out


def run_c4(args):
    """Out-of-core fly-through: a uint8 layered-blob volume streamed brick by
    brick into a page-locked host store (LZ4-compressed in 16 KiB chunks,
    decoded on the GPU when paged; --no-compress: raw), 256^3 bricks, 2
    ghosts, 6 levels, a device slot pool holding 3/8 of the volume (the
    96 GiB : 256 GiB ratio), a 120-frame Bezier fly-through at 1920x1080 with
    a 256-entry 1D TF.  Default 4096x4096x2048 (1/8 of the volume);
    --size 8192: the full 8192x8192x4096 volume.  One step = one pass over the
    path.
    value: frames/s of paint (page-in of missing bricks + render), wall clock
    per frame; e2e: the same with every frame read back into page-locked host
    memory.  Error: GPU frame vs the FP64 oracle on the level the frame
    resolved, on a seeded pixel sample."""
    import numpy as np
    import torch
    from imagevis3d_gb300 import Renderer, workloads
    from oracle import orc
    size = (4096, 4096, 2048) if args.size == 1024 else (args.size, args.size, args.size // 2)
    wl = workloads.config4(size=size, frames=args.frames)
    vol_bytes = size[0] * size[1] * size[2]
    pool = int(args.pool_gib * (1 << 30)) if args.pool_gib > 0 else vol_bytes * 3 // 8
    r = Renderer()
    t0 = time.perf_counter()
    codec = 0 if args.no_compress else {"lz4": 3, "zlib": 1}[args.codec]
    r.loadSyntheticOutOfCore(wl.synth, pool, compression=codec, brick_order=args.brick_order, **wl.brick)
    build_s = time.perf_counter() - t0
    info = r.datasetInfo()
    r.resize((wl.width, wl.height))
    r.set1DTrans(wl.tf)
    r.setValueRange(*wl.value_range)
    r.setSampleRateModifier(wl.spv)
    host = torch.empty((wl.height, wl.width, 4), dtype=torch.uint8).pin_memory()

    def frame(view, proj, readback):
        t1 = time.perf_counter()
        r.setView(view, proj)
        r.paint()
        if readback:
            r.readFramebuffers(0, 1, host)
        return time.perf_counter() - t1, r.stats()

    # warm-up: the first frames of the path, synchronously
    for view, proj in wl.views[:args.warmup]:
        frame(view, proj, False)
    frames = len(wl.views)
    host_all = torch.empty((frames, wl.height, wl.width, 4), dtype=torch.uint8).pin_memory()
    passes = []
    clk = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clk.start()
    for _ in range(args.steps):
        t1 = time.perf_counter()
        lod, miss, paged = r.paintPath(wl.views)
        wall = time.perf_counter() - t1
        st = r.stats()
        passes.append((wall, lod, miss, paged, st))
    # end to end: the path with every frame captured into page-locked memory
    # as it completes (the read-back of frame i overlaps frames i + 1 ..)
    t1 = time.perf_counter()
    lod_e, miss_e, paged_e = r.paintPath(wl.views, capture=host_all)
    e2e_wall = time.perf_counter() - t1
    e2e_h2d = r.stats()["h2d_bytes"]
    clocks = clk.stop()
    # the same path painted frame by frame (synchronous paging, no overlap)
    seq = [frame(v, p, False) for v, p in wl.views]
    # error at the level each sampled frame resolved
    err = []
    cpu_pix_s = None
    levels = {}
    if not args.no_cpu:
        for fi in (len(wl.views) // 4, len(wl.views) // 2):
            view, proj = wl.views[fi]
            _, st = frame(view, proj, True)
            img = host.numpy().astype(np.float64) / 255.0
            lod = st["lod"]
            ld = info["lod_dims"][lod]
            if ld[0] * ld[1] * ld[2] > 40e9:
                continue  # the level does not fit the oracle's host memory
            if lod not in levels:
                levels[lod] = level_from_bricks(r, lod)
            lvl = levels[lod]
            rng = np.random.default_rng(workloads.SEED + fi)
            pix = rng.integers(0, wl.width * wl.height, 4096)
            tc = time.perf_counter()
            ref, _ = orc.render(lvl, view, proj, wl.width, wl.height, wl.tf, spv=wl.spv,
                                value_range=wl.value_range, pixels=pix, threads=orc.max_threads(),
                                extent=tuple(np.array(size, np.float64) / max(size)))
            cpu_pix_s = len(pix) / (time.perf_counter() - tc)
            got = img.reshape(-1, 4)[pix]
            d = np.abs(got - ref)
            err.append({"frame": fi, "lod": lod, "max": float(d.max()), "rms": float(np.sqrt((d * d).mean()))})
        levels.clear()
    r.cleanup()
    walls = [p[0] for p in passes]
    fps = frames * len(passes) / sum(walls)
    misses = sum(int(p[2].sum()) for p in passes)
    paged = sum(int(p[3].sum()) for p in passes)
    page_ms = sum(p[4]["page_ms"] for p in passes)
    paged_comp = sum(int(p[4]["bytes_paged_compressed"]) for p in passes)
    host_copies = sum(int(p[4]["host_copies"]) for p in passes)
    h2d = paged_comp if info["compression"] else paged
    lod_hist = {}
    for p in passes:
        for l in p[1]:
            lod_hist[str(int(l))] = lod_hist.get(str(int(l)), 0) + 1
    seq_wall = sum(w for w, _ in seq)
    seq_kernel = sum(st["kernel_ms"] for _, st in seq)
    out = {
        "metric": "out-of-core fly-through frames/s, brick misses/frame, host->device GB/s",
        "value": fps, "unit": "frames/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * sum(walls) / len(walls), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded blob volume, streamed from seed)",
        "config": {"workload": wl.name, "volume_bytes": vol_bytes, "host_store_bytes": info["host_bytes"],
                   "host_store_raw_bytes": info["host_raw_bytes"],
                   "store_brick_order": ["scanline", "Morton", "Hilbert", "random"][args.brick_order],
                   "store_compression": ({3: "lz4", 1: "zlib"}[info["compression"]] + " (16 KiB chunks, decoded on "
                                         "the GPU)") if info["compression"] else "none",
                   "device_pool_bytes": pool, "device_slots": info["device_slots"], "bricks": info["total_bricks"],
                   "lods": info["lod_count"], "frames_per_step": frames, "width": wl.width, "height": wl.height,
                   "l2": "volume and pool larger than L2", "step": "gbvr_paint_path over the 120-frame path"},
        "misses_per_frame": misses / (frames * len(passes)),
        "paged_bytes_per_frame": paged / (frames * len(passes)),
        "h2d_gbps": h2d / (page_ms / 1000.0) / 1e9 if page_ms > 0 else None,
        "paged_raw_gbps": paged / (page_ms / 1000.0) / 1e9 if page_ms > 0 else None,
        "paged_compressed_bytes_per_frame": paged_comp / (frames * len(passes)),
        "host_copies_per_frame": host_copies / (frames * len(passes)),
        "store_ratio": info["host_raw_bytes"] / max(info["host_bytes"], 1),
        "lod_frames": lod_hist,
        "first_pass_fps": frames / walls[0], "last_pass_fps": frames / walls[-1],
        "per_frame_paint_fps": frames / seq_wall, "per_frame_render_fps_kernel_only": frames / (seq_kernel / 1000.0),
        "pipeline_vs_per_frame": fps / (frames / seq_wall),
        "e2e": {"value": frames / e2e_wall, "unit": "frames/s", "h2d_bytes_per_step": int(e2e_h2d),
                "d2h_bytes_per_step": frames * wl.width * wl.height * 4,
                "how": "gbvr_paint_path_capture: the path with each frame's RGBA8 pixels copied into page-locked "
                       "host memory as soon as the frame is done"},
        "image_error_at_resolved_lod": err,
        "cpu_baseline": {"value": cpu_pix_s / (wl.width * wl.height) if cpu_pix_s else None, "unit": "frames/s",
                         "cores": orc.max_threads(), "kind": "port",
                         "sample": "4096 seeded pixels of one frame at its resolved level"},
        "build_s": build_s, "gpu_launches": 2 * frames * (len(passes) + 2), "clocks": clocks,
    }
    print(json.dumps(out))
    return 0


def serving_run(nreq, plain_requests, max_batch, err_requests=6, seed_offset=5, slots=3, pool_fraction=0.0):
    """Serving mix: Poisson arrivals of render requests over 12 resident
    datasets (64^3 .. 1024^3, uint8 / uint16 / float32), image sizes in
    {256^2, 512^2, 1280x720, 1920x1080}, a random 1D or 2D TF preset and a
    random camera per request.  Capacity is measured first with a burst; the
    Poisson stream then runs at 70% of it.  The plain per-request path (one
    renderer paint + readback per request) is timed on the same requests.
    The image error against the FP64 oracle is taken on `err_requests`
    requests of the datasets up to 384^3 (their RGBA8 images as served, so the
    8-bit rounding is included).  `slots` batches are in flight at once; the
    launch shapes come from the server's autotuner; pool_fraction > 0 caps the
    device brick-pool memory at that fraction of all datasets' pools
    (admission by memory: pools evicted and uploaded on demand).  Returns a
    dict."""
    import threading as th
    import numpy as np
    from imagevis3d_gb300 import (GBVR_RM_1DTRANS, GBVR_RM_2DTRANS, Renderer, Server, orbit_camera,
                                  synth_params, workloads)
    rng = np.random.default_rng(workloads.SEED + seed_offset)
    sizes_vol = [64, 96, 128, 192, 256, 320, 384, 512, 640, 768, 896, 1024]
    dtypes = [np.uint8, np.uint16, np.float32]
    specs = []
    for i, n in enumerate(sizes_vol):
        dt = dtypes[i % 3]
        scale, vmax = {np.uint8: (255.0, 255.0), np.uint16: (2600.0, 4095.0), np.float32: (1.0, 1.0)}[dt]
        specs.append(synth_params((n, n, n), dt, 500 + i, 24, (0.03 * n, 0.09 * n), (0.3, 1.0), scale,
                                  noise_kind=2, noise_amp=0.02 * scale, vmax=vmax))
    img_sizes = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]
    pools = []
    if pool_fraction > 0:
        # the datasets' pool sizes, from an unbudgeted server's resident bytes
        with Server(max_batch=max_batch, fb_budget_bytes=64 << 20, slots=1) as probe:
            prev = 0
            for sp in specs:
                probe.add_synthetic(sp, brick_size=256, overlap=2, layouts=1)
                cur = probe.stats()["resident_bytes"]
                pools.append(cur - prev)
                prev = cur
    budget = max(max(pools), int(pool_fraction * sum(pools))) if pools else 0
    srv = Server(max_batch=max_batch, fb_budget_bytes=1 << 30, slots=slots, device_pool_bytes=budget)
    ds, presets = [], []
    for i, sp in enumerate(specs):
        d = srv.add_synthetic(sp, brick_size=256, overlap=2, layouts=1)
        ds.append(d)
        vmax = float(sp.vmax) if sp.dtype != 2 else 1.0
        t1 = workloads.tf1d_seeded(256, 700 + i, 0.3 * vmax, vmax)
        t2 = workloads.tf2d_seeded(256, 128, 800 + i, zero_cols=60)
        presets.append([(srv.add_tf(d, GBVR_RM_1DTRANS, t1), GBVR_RM_1DTRANS, t1),
                        (srv.add_tf(d, GBVR_RM_2DTRANS, t2, grad_max=0.05), GBVR_RM_2DTRANS, t2)])
    reqs = []
    for _ in range(nreq):
        di = int(rng.integers(0, len(ds)))
        pi = int(rng.integers(0, 2))
        w, h = img_sizes[int(rng.integers(0, 4))]
        cam = orbit_camera(float(rng.uniform(0, 360)), float(rng.uniform(-45, 45)),
                           float(rng.uniform(1.8, 3.0)) * workloads.DIAG, 45.0, w, h)
        reqs.append((di, pi, w, h, cam))

    def run_stream(arrivals, outs=None):
        tickets = []
        q = []
        lock = th.Lock()
        finished = th.Event()

        def waiter():
            k = 0
            while k < len(arrivals):
                with lock:
                    t = q[k] if k < len(q) else None
                if t is None:
                    time.sleep(0.0002)
                    continue
                srv.wait(t)
                k += 1
            finished.set()
        wt = th.Thread(target=waiter, daemon=True)
        wt.start()
        t0 = time.perf_counter()
        for j, ((di, pi, w, h, cam), ta) in enumerate(zip(reqs, arrivals)):
            delay = ta - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            out = outs[j] if outs is not None and j in outs else None
            t = srv.submit(ds[di], presets[di][pi][0], w, h, cam[0], cam[1], out=out)
            with lock:
                q.append(t)
        finished.wait()
        return time.perf_counter() - t0

    tune = srv.autotune(512, 512, 16)
    # warm-up and capacity (burst)
    srv.reset_stats()
    run_stream([0.0] * min(200, nreq))
    srv.reset_stats()
    wall = run_stream([0.0] * nreq)
    burst = srv.stats()
    capacity = burst["completed"] / wall
    # Poisson arrivals at 70% of capacity; the images of a few small requests kept for the error check
    rate = 0.7 * capacity
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq)).tolist()
    err_idx = [j for j, rq in enumerate(reqs) if sizes_vol[rq[0]] <= 384][:err_requests]
    outs = {j: np.zeros((reqs[j][3], reqs[j][2], 4), np.uint8) for j in err_idx}
    srv.reset_stats()
    wall = run_stream(arrivals, outs)
    st = srv.stats()
    srv.close()
    # plain per-request path: one renderer per dataset, paint + readback
    plain_fps, lat = None, []
    if plain_requests > 0:
        rends = []
        for i, sp in enumerate(specs):
            r = Renderer()
            r.loadSynthetic(sp, brick_size=256, overlap=2)
            rends.append(r)
        sample = reqs[:min(len(reqs), plain_requests)]
        t0 = time.perf_counter()
        for di, pi, w, h, cam in sample:
            t1 = time.perf_counter()
            r = rends[di]
            _, mode, tf = presets[di][pi]
            r.resize((w, h))
            r.setRenderMode(mode)
            if mode == GBVR_RM_1DTRANS:
                r.set1DTrans(tf)
            else:
                r.set2DTrans(tf, 0.05)
            r.setView(*cam)
            r.paint()
            r.readFramebuffer(0)
            lat.append((time.perf_counter() - t1) * 1000.0)
        plain_fps = len(sample) / (time.perf_counter() - t0)
        for r in rends:
            r.cleanup()
        lat.sort()
    # error of served images against the FP64 oracle (pixel subsets; the
    # servers's default value range: [0, max] for integers, [min, max] for float32)
    err = None
    if err_idx:
        from oracle import orc
        worst_max, sq, n = 0.0, 0.0, 0
        vols = {}
        prng = np.random.default_rng(workloads.SEED + 55)
        for j in err_idx:
            di, pi, w, h, cam = reqs[j]
            if di not in vols:
                vols[di] = orc.synth_blobs(specs[di])
            vol = vols[di]
            _, mode, tf = presets[di][pi]
            vr = (float(vol.min()), float(vol.max())) if vol.dtype == np.float32 else (0.0, max(1.0, float(vol.max())))
            img = outs[j].reshape(-1, 4).astype(np.float64) / 255.0
            cov = np.flatnonzero(img[:, 3] > 0.02)
            pix = np.concatenate([prng.choice(cov, min(300, cov.size), replace=False) if cov.size else
                                  np.zeros(0, np.int64), prng.integers(0, w * h, 100)])
            kw = dict(mode=1, grad_max=0.05) if mode == GBVR_RM_2DTRANS else dict(mode=0)
            ref, _ = orc.render(vol, cam[0], cam[1], w, h, tf, value_range=vr, pixels=pix, **kw)
            d = np.abs(np.clip(img[pix], 0, 1) - np.clip(ref, 0, 1))
            worst_max = max(worst_max, float(d.max()))
            sq += float((d * d).sum())
            n += d.size
        err = {"max": worst_max, "rms": math.sqrt(sq / n), "requests": len(err_idx),
               "pixels": n // 4, "tol_max": 2 / 255, "tol_rms": 0.5 / 255,
               "note": "RGBA8 images as served (8-bit rounding included), seeded pixel subsets"}
    return {
        "frames_per_s": st["frames_per_s"], "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "max_ms": st["max_ms"],
        "mean_batch": st["mean_batch"], "requests": nreq, "arrival_rate_per_s": rate,
        "burst_capacity_fps": capacity, "burst_p99_ms": burst["p99_ms"], "plain_per_request_fps": plain_fps,
        "plain_p50_ms": lat[len(lat) // 2] if lat else None,
        "plain_p99_ms": lat[min(len(lat) - 1, int(0.99 * (len(lat) - 1) + 0.5))] if lat else None,
        "serving_vs_plain": capacity / plain_fps if plain_fps else None, "max_batch": max_batch, "image_error_vs_fp64": err,
        "slots": slots, "batches": st["batches"], "overlapped_batch_pairs": st["overlapped"],
        "checked_batch_pairs": st["overlap_checked"], "burst_overlapped_pairs": burst["overlapped"],
        "device_pool_bytes": budget, "pool_uploads": st["uploads"], "pool_evictions": st["evictions"],
        "pool_upload_bytes": st["upload_bytes"], "all_pools_bytes": sum(pools) if pools else None,
        "autotune": tune,
    }


def run_c5(args):
    """Serving mix at full length (10k requests by default); prints one JSON line of its own."""
    sv = serving_run(args.requests, args.plain_requests, args.max_batch, slots=args.slots)
    # the same stream under a brick-pool budget of half the datasets' pools
    svm = serving_run(min(args.requests, 2000), 0, args.max_batch, err_requests=0, slots=args.slots,
                      pool_fraction=0.5) if args.pool_pass else None
    out = {
        "metric": "serving frames/s & p50/p99 latency (Poisson arrivals, continuous batching)",
        "value": sv["frames_per_s"], "unit": "frames/s", "n_gpus": 1, "steps": args.requests, "warmup": 200,
        "ms_per_step": 1000.0 / max(sv["frames_per_s"], 1e-9), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded blob volumes)",
        "config": {"workload": "c5_serving_12_datasets_%d_requests" % args.requests,
                   "datasets": "64^3..1024^3 u8/u16/f32",
                   "image_sizes": [(256, 256), (512, 512), (1280, 720), (1920, 1080)],
                   "arrival_rate_per_s": sv["arrival_rate_per_s"], "max_batch": args.max_batch},
    }
    out.update({k: v for k, v in sv.items() if k not in ("frames_per_s", "arrival_rate_per_s")})
    if svm:
        out["memory_budget_pass"] = {k: svm[k] for k in ("frames_per_s", "p50_ms", "p99_ms", "burst_capacity_fps",
                                                          "device_pool_bytes", "all_pools_bytes", "pool_uploads",
                                                          "pool_evictions", "pool_upload_bytes", "requests")}
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--views", type=int, default=64)
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-seconds", type=float, default=8.0)
    ap.add_argument("--cpu-volume", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-texture", action="store_true")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4", "c5"])
    ap.add_argument("--frames", type=int, default=120)
    ap.add_argument("--pool-gib", type=float, default=0.0)
    ap.add_argument("--no-compress", action="store_true", help="c4: raw host brick store")
    ap.add_argument("--codec", default="lz4", choices=["lz4", "zlib"], help="c4: codec of the host brick store")
    ap.add_argument("--brick-order", type=int, default=0, choices=[0, 1, 2, 3],
                    help="c4: host store brick order: 0 scanline, 1 Morton, 2 Hilbert, 3 random")
    ap.add_argument("--requests", type=int, default=10000)
    ap.add_argument("--plain-requests", type=int, default=600)
    ap.add_argument("--max-batch", type=int, default=64)
    ap.add_argument("--slots", type=int, default=3, help="serving: batches in flight")
    ap.add_argument("--no-tune-ex", action="store_true", help="c2: skip the extended autotuner")
    ap.add_argument("--pool-pass", type=int, default=1, help="c5: also run under a half-size brick-pool budget")
    ap.add_argument("--serve-requests", type=int, default=400,
                    help="c2: requests of the short serving run giving p50/p99 (0: skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "c3" and args.impl == "ours":
        return run_c3(args)
    if args.workload == "c4" and args.impl == "ours":
        return run_c4(args)
    if args.workload == "c5" and args.impl == "ours":
        return run_c5(args)

    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from imagevis3d_gb300 import (GBVR_RM_1DTRANS, GBVR_RM_MIP, GBVR_SAMPLER_SW, GBVR_SAMPLER_TEX, Renderer,
                                  synth_volume, workloads)
    from imagevis3d_gb300.replicas import shard

    wl = workloads.config2(size=args.size, nviews=args.views)
    # replicas: each rank renders its own share of the orbit (no exchange)
    mine = shard(len(wl.views), rank, world)
    views = [wl.views[i] for i in mine]
    r = Renderer()
    # the GPU UVF build of the volume (device time per phase), measured on the
    # second build in the process: the first also loads every build kernel
    # (lazy module loading) and grows the stream-ordered pool, once
    r.loadSynthetic(wl.synth, **wl.brick, build_texture=False, layouts=4)
    build_first = r.buildStats()
    r.loadSynthetic(wl.synth, **wl.brick, build_texture=not args.no_texture, layouts=4)
    build = r.buildStats()
    r.resize((wl.width, wl.height))
    r.set1DTrans(wl.tf)
    r.setValueRange(*wl.value_range)
    r.setSampleRateModifier(wl.spv)
    info = r.datasetInfo()
    # launch shape picked by the autotuner on this batch (setup, untimed)
    tune = r.autotune(views)

    def barrier():
        if dist is not None:
            dist.barrier()

    def maxover(x):
        if dist is None:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # ---- device-resident batched throughput (value) ----
    for _ in range(args.warmup):
        r.paintBatch(views)
    vis = [v for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
    clocks = ClockSampler(vis[local] if local < len(vis) else local)
    barrier()
    clocks.start()
    kernel_ms, step_ms, samples, brick_bytes = [], [], 0, 0
    for _ in range(args.steps):
        r.paintBatch(views)
        st = r.stats()
        kernel_ms.append(st["kernel_ms"])
        step_ms.append(st["gpu_ms"])
        samples += st["samples"]
        brick_bytes += st["brick_bytes"]
    barrier()
    clk = clocks.stop()
    # algorithmic bytes: distinct non-empty 4^3 macro-cells each view samples
    # (one untimed pass with the per-cell bitmap enabled)
    r.setStatsLevel(2)
    r.paintBatch(views)
    st2 = r.stats()
    # the 8-view orbit the committed ncu capture rendered (bench.py --views 8)
    r.paintBatch(workloads.config2(size=args.size, nviews=8).views)
    st8 = r.stats()
    r.setStatsLevel(1)
    cell_bytes_per_launch = st2["cell_bytes"]
    dev_s = maxover(sum(step_ms) / 1000.0)
    frames_total = len(wl.views) * args.steps  # all ranks
    value = frames_total / dev_s
    ksec = sum(kernel_ms) / 1000.0
    achieved = None
    st_last = st  # the last timed step

    # ---- per-view plain kernel (64 launches) ----
    plain_ms = []
    for _ in range(2):
        r.paintViews(views)
    for _ in range(args.steps):
        r.paintViews(views)
        plain_ms.append(r.stats()["gpu_ms"])
    plain_fps = len(views) * args.steps / (sum(plain_ms) / 1000.0)
    # the drop-in single-view paint (a one-view persistent launch), device time
    paint_ms = []
    for v, p in views:
        r.setView(v, p)
        r.paint()
        paint_ms.append(r.stats()["gpu_ms"])
    paint_fps = len(views) / (sum(paint_ms) / 1000.0)

    # ---- texture-hardware trilinear, same batch ----
    tex_fps = None
    tune_tex = None
    if not args.no_texture:
        r.setSampler(GBVR_SAMPLER_TEX)
        tune_tex = r.autotune(views)
        for _ in range(2):
            r.paintBatch(views)
        tms = []
        for _ in range(args.steps):
            r.paintBatch(views)
            tms.append(r.stats()["gpu_ms"])
        tex_fps = len(views) * args.steps / (sum(tms) / 1000.0)
        r.setSampler(GBVR_SAMPLER_SW)
        r.setLaunchShape(tune["tile_w"], tune["ctas_per_sm"])

    # ---- the same batch in MIP mode, and with both bounding boxes drawn ----
    def batch_fps():
        for _ in range(2):
            r.paintBatch(views)
        ms_ = []
        for _ in range(args.steps):
            r.paintBatch(views)
            ms_.append(r.stats()["gpu_ms"])
        return len(views) * args.steps / (sum(ms_) / 1000.0)

    r.setRenderMode(GBVR_RM_MIP)
    mip_fps = batch_fps()
    r.setRenderMode(GBVR_RM_1DTRANS)
    r.setGlobalBBox(True)
    r.setLocalBBox(True)
    bbox_fps = batch_fps()
    r.setGlobalBBox(False)
    r.setLocalBBox(False)

    # ---- end to end through the public API with host buffers ----
    # (the caller's destination is page-locked host memory, one copy per step)
    import torch
    host_fb = torch.empty((len(views), wl.height, wl.width, 4), dtype=torch.uint8, pin_memory=True)
    r.paintBatch(views)
    r.readFramebuffers(0, len(views), host_fb)
    # synchronous: paint, then read back, step after step
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r.paintBatch(views)
        r.readFramebuffers(0, len(views), host_fb)
    barrier()
    e2e_sync = frames_total / maxover(time.perf_counter() - t0)
    h2d = r.stats()["h2d_bytes"]
    d2h = len(views) * wl.width * wl.height * 4
    # pipelined (the e2e value): step i renders into framebuffer set i % 2
    # while step i - 1's frames are read back into their own host buffer; the
    # host waits for each step's read-back (a consumer could use the frames
    # then) while the next render runs
    host2 = [host_fb, torch.empty_like(host_fb).pin_memory()]
    for i in range(2):
        r.paintBatchAsync(views, i)
    r.waitAsync()
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        r.paintBatchAsync(views, i % 2)
        if i > 0:
            r.readFramebuffersAsync((i - 1) % 2, host2[(i - 1) % 2])
            r.waitRead((i - 1) % 2)
    r.readFramebuffersAsync((args.steps - 1) % 2, host2[(args.steps - 1) % 2])
    r.waitAsync()
    barrier()
    e2e_s = maxover(time.perf_counter() - t0)
    e2e = frames_total / e2e_s
    del host_fb, host2

    # per-view drop-in end to end: paint + readback one view at a time
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps // 2)):
        for v, p in views:
            r.setView(v, p)
            r.paint()
            r.readFramebuffer(0)
    e2e_plain = len(views) * max(1, args.steps // 2) / (time.perf_counter() - t0)

    # ---- the extended autotuner (untimed, after every measurement above): launch
    # shape x brick size (the dataset rebuilt from its finest level, same pixels)
    # x samples per inner-loop step.  The headline keeps the configuration's 256^3
    # bricks; this reports what the tuner would choose and the spread.
    tune_ex = None
    if not args.no_tune_ex:
        r.setLaunchShape(8, 0)
        tune_ex = r.autotuneEx(views, brick_sizes=(128, 256, 512), samples_per_step=(1, 4))
        tune_ex["gain_vs_default"] = tune_ex["default_ms"] / tune_ex["best_ms"] if tune_ex["best_ms"] > 0 else None
    r.cleanup()
    # ---- short serving run (the metric's p99): Poisson arrivals at 70% of capacity ----
    sv = serving_run(args.serve_requests, 100, args.max_batch, err_requests=4) if args.serve_requests > 0 else None

    out = None
    if rank == 0:
        pk = peaks()
        peak = pk["hbm_gbs"] if pk else 6800.0
        cpu = None
        err = None
        cpu_build = None
        if not args.no_cpu:
            from oracle import orc
            vol = synth_volume(wl.synth)
            threads = orc.max_threads()
            v0, p0 = wl.views[0]
            pr, sr, n, ref, pix, el = cpu_sample(wl, vol, v0, p0, args.cpu_seconds, threads, 7)
            pr1, sr1, n1, _, _, el1 = cpu_sample(wl, vol, v0, p0, args.cpu_seconds / 3.0, 1, 8)
            cpu = {"value": pr / (wl.width * wl.height), "unit": "frames/s", "cores": threads,
                   "kind": "port", "gsamples_per_s": sr / 1e9,
                   "value_1core": pr1 / (wl.width * wl.height), "gsamples_per_s_1core": sr1 / 1e9,
                   "sample": "%d seeded pixels of view 0 (%.1f s, FP64 oracle, %d threads; 1 thread: %d "
                             "pixels in %.1f s); frames/s = pixels/s / (%d*%d)" %
                             (n, el, threads, n1, el1, wl.width, wl.height)}
            # the CPU UVF build restatement on the same generator at 1/8 of the voxels
            # (512^3), all threads and 1 thread, scaled to the full volume by voxel count
            from oracle import scenes
            small = orc.synth_blobs(scenes.config2(size=args.size // 2, nviews=1).synth)
            scale = float(vol.size) / float(small.size)
            tb_all, ph_all = orc.uvf_build_timed(small, threads=threads)
            tb_1, ph_1 = orc.uvf_build_timed(small, threads=1)
            del small
            cpu_build = {"kind": "port", "cores": threads, "seconds": tb_all * scale, "seconds_1core": tb_1 * scale,
                         "phases_s": {k: v * scale for k, v in ph_all.items()},
                         "phases_s_1core": {k: v * scale for k, v in ph_1.items()},
                         "sample": "the oracle's CPU build (pyramid, bricks + min/max, 1D and 2D histograms) of "
                                   "the %d^3 volume of the same generator, times scaled by voxel count x%.0f"
                                   % (args.size // 2, scale)}
            # image error of the GPU frame on the same pixels
            r2 = Renderer(float_fb=True)
            r2.loadSynthetic(wl.synth, **wl.brick)
            r2.resize((wl.width, wl.height))
            r2.set1DTrans(wl.tf)
            r2.setValueRange(*wl.value_range)
            r2.setSampleRateModifier(wl.spv)
            r2.setView(v0, p0)
            r2.paint()
            img = r2.readFramebuffer(0, as_float=True).reshape(-1, 4)[pix]
            r2.cleanup()
            d = np.abs(img - ref)
            err = {"max": float(d.max()), "rms": float(np.sqrt((d * d).mean())),
                   "pixels": int(pix.size), "tol_max": 2 / 255, "tol_rms": 0.5 / 255}
        gs = samples / (sum(kernel_ms) / 1000.0) / 1e9
        achieved = cell_bytes_per_launch / (ksec / args.steps) / 1e9
        # traffic and issue: the committed 8-view ncu capture, scaled to this
        # launch by the algorithmic bytes / samples measured here on both
        prof = profile_counters()
        traffic = issue = None
        if prof and st8["cell_bytes"] > 0 and st8["samples"] > 0:
            dram8 = prof.get("dram__bytes_read.sum", 0.0) + prof.get("dram__bytes_write.sum", 0.0)
            traffic = dram8 * cell_bytes_per_launch / st8["cell_bytes"]
            inst = prof.get("smsp__inst_executed.sum", 0.0) * st_last["samples"] / st8["samples"]
            sm_hz = (clk.get("sm_mhz") or 2070.0) * 1e6
            nsm = int(prof.get("device__attribute_multiprocessor_count", 152))
            issue_peak = 4.0 * nsm * sm_hz  # one warp instruction per SMSP per cycle, 4 SMSPs per SM
            issue_ach = inst / (ksec / args.steps)
            issue = {"bound": "issue", "achieved": issue_ach, "peak": issue_peak, "unit": "warp-inst/s",
                     "frac": issue_ach / issue_peak,
                     "capture_issue_active_pct": prof.get("smsp__issue_active.avg.pct_of_peak_sustained_active"),
                     "capture_threads_per_inst": prof.get("smsp__thread_inst_executed_per_inst_executed.ratio"),
                     "how": "warp instructions of the 8-view capture x (samples here / samples of the 8 views "
                            "here), over this launch's kernel time; peak = 4 x SMs x SM clock"}
        bgbps = build["total_bytes"] / (build["total_ms"] / 1000.0) / 1e9 if build["total_ms"] > 0 else None
        uvf_build = {
            "workload": "GPU UVF build of the %d^3 uint16 volume: %d LODs, 256^3 bricks with 2 ghosts, %d layout "
                        "copies, macro-cell min/max, per-brick min/max, 1D and 2D histograms (synthesis and "
                        "textures excluded)" % (args.size, build["lod_count"], build["layout_copies"]),
            "ms": build["total_ms"], "ms_first_build": build_first["total_ms"], "bytes": build["total_bytes"],
            "gbps": bgbps,
            "roofline": {"bound": "hbm", "achieved": bgbps, "peak": peak, "unit": "GB/s",
                         "frac": bgbps / peak if bgbps else None},
            "phases_ms": {k[:-3]: build[k] for k in ("pyramid_ms", "cells_ms", "bricks_ms", "minmax_ms",
                                                     "hist1d_ms", "hist2d_ms")},
            "phases_bytes": {k[:-6]: build[k] for k in ("pyramid_bytes", "cells_bytes", "bricks_bytes",
                                                        "minmax_bytes", "hist1d_bytes", "hist2d_bytes")},
            "cpu_baseline": cpu_build,
        }
        out = {
            "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded Philox blob volume)",
            "config": {"workload": wl.name, "volume": "%d^3 uint16 (12-bit)" % args.size,
                       "bricks": "256^3 incl. 2 ghosts, %d bricks at LOD 0, %d LODs" %
                                 (int(np.prod(info["lod_bricks"][0])), info["lod_count"]),
                       "views": len(wl.views), "width": wl.width, "height": wl.height,
                       "samples_per_voxel": wl.spv, "lod": 0, "tf_entries": 4096,
                       "sampler": "fp32 software trilinear",
                       "brick_layouts": "4x4x4-blocked copy (plus the x-fastest copy)",
                       "empty_skipping": "bricks + 4^3 macro-cells with a distance field",
                       "l2": "inputs larger than L2 (brick pool %.2f GB)" % (info["device_bytes"] / 1e9),
                       "parallelism": "replicas" if world > 1 else "1 GPU"},
            "gsamples_per_s": gs,
            "per_view_plain_fps": plain_fps,
            "per_view_paint_fps": paint_fps,
            "batched_vs_per_view": value / plain_fps,
            "texture_trilinear_fps": tex_fps,
            "mip_fps": mip_fps,
            "with_bboxes_fps": bbox_fps,
            "autotune": {"sw": tune, "tex": tune_tex, "extended": tune_ex},
            "e2e_per_view_fps": e2e_plain,
            "image_error_vs_fp64": err,
            "e2e": {"value": e2e, "unit": "frames/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "how": "gbvr_paint_batch_async + gbvr_read_framebuffers_async into page-locked host memory, "
                           "read-back of step i overlapping the render of step i + 1; every step's frames read back"},
            "e2e_sync_fps": e2e_sync,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_render_persistent_u<uint16,1D,SW>",
                         "bytes_per_launch": cell_bytes_per_launch,
                         "bytes_rule": "sum over views of distinct non-empty 4^3 macro-cells sampled x 4^3 x 2 B",
                         "brick_bytes_per_launch": brick_bytes / args.steps,
                         "kernel_ms": 1000.0 * ksec / args.steps,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if pk else "fallback",
                         "traffic_how": "DRAM bytes of the committed 8-view ncu capture x (algorithmic bytes here / "
                                        "algorithmic bytes of the same 8 views here)",
                         "issue": issue},
            "cpu_baseline": cpu,
            "uvf_build": uvf_build,
            "p50_ms": sv["p50_ms"] if sv else None,
            "p99_ms": sv["p99_ms"] if sv else None,
            "serving": sv,
            "gpu_launches": 2 * args.steps,  # per step: the background fill and the persistent raycast
            "clocks": clk,
            "stats_last_step": {k: st_last[k] for k in ("samples", "bricks_touched", "bricks_skipped",
                                                         "brick_bytes")},
        }
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
