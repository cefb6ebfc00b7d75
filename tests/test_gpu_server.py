"""Serving loop: datasets and TF presets, requests from a burst and one at a
time; every image equals the same request rendered alone, in a server with
another slot count, launch shape or memory budget, and the same view rendered
through the renderer API, bit for bit.  Batches overlap on the device;
datasets are evicted and uploaded again under a brick-pool budget; a failed
launch fails its batch and the worker goes on."""
import numpy as np
import pytest

from imagevis3d_gb300 import (GBVR_RM_1DTRANS, GBVR_RM_2DTRANS, GBVR_RM_ISOSURFACE, GBVR_RM_MIP, GbvrError,
                              Renderer, Server, orbit_camera, synth_params, workloads)

pytestmark = pytest.mark.gpu

SIZES = [(64, 48), (96, 96), (160, 90), (40, 40)]


@pytest.fixture(scope="module")
def setup(orc):
    vols = [
        synth_params((96, 96, 96), np.uint8, 1, 6, (4.0, 12.0), (0.4, 1.0), 255.0, noise_kind=1, noise_amp=3.0,
                     vmax=255.0),
        synth_params((128, 112, 100), np.uint16, 2, 12, (5.0, 15.0), (0.3, 1.0), 2600.0, noise_kind=2,
                     noise_amp=20.0, vmax=4095.0, bg_freq=1.0, bg_level=0.15, bg_amp=0.1),
        synth_params((80, 80, 80), np.float32, 3, 8, (4.0, 14.0), (0.3, 1.0), 1.0),
    ]
    hosts = [orc.synth_blobs(v) for v in vols]
    tfs = [
        (GBVR_RM_1DTRANS, workloads.tf1d_seeded(256, 5, 60.0, 255.0), {}),
        (GBVR_RM_1DTRANS, workloads.tf1d_seeded(4096, 6, 900.0, 4095.0), {}),
        (GBVR_RM_2DTRANS, workloads.tf2d_seeded(128, 64, 7, zero_cols=10), {"grad_max": 0.08}),
        (GBVR_RM_1DTRANS, workloads.tf1d_seeded(512, 8, 0.2, 1.0), {}),
        (GBVR_RM_ISOSURFACE, None, {"iso": 1200.0, "iso_rgb": (0.9, 0.6, 0.3)}),
        # MIP on uint8 next to 1D on uint16: distinct launch groups
        (GBVR_RM_MIP, workloads.tf1d_seeded(256, 9, 40.0, 255.0), {}),
    ]
    owners = [0, 1, 1, 2, 1, 0]
    return vols, hosts, tfs, owners


def _requests(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        tf = int(rng.integers(0, 6))
        w, h = SIZES[int(rng.integers(0, len(SIZES)))]
        cam = orbit_camera(float(rng.uniform(0, 360)), float(rng.uniform(-40, 40)),
                           float(rng.uniform(1.6, 3.0)) * workloads.DIAG, 45.0, w, h)
        out.append((tf, w, h, cam, float(rng.choice([1.0, 1.5]))))
    return out


def test_mix_alone_and_renderer_agree(setup):
    vols, hosts, tfs, owners = setup
    reqs = _requests(36, 11)
    with Server(max_batch=8, fb_budget_bytes=4 << 20) as srv:
        ds = [srv.add_synthetic(v, brick_size=64, overlap=2) for v in vols]
        tf_ids = [srv.add_tf(ds[owners[i]], m, t, **kw) for i, (m, t, kw) in enumerate(tfs)]
        # a burst: everything submitted before anything is waited for
        tickets = [srv.submit(ds[owners[tf]], tf_ids[tf], w, h, cam[0], cam[1], spv) for tf, w, h, cam, spv in reqs]
        mixed = [srv.wait(t) for t in tickets]
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["batches"] < len(reqs) and st["mean_batch"] > 1.5
        assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
        assert max(r["batch_size"] for _, r in mixed) <= 8
        # one at a time
        alone = []
        for tf, w, h, cam, spv in reqs[:12]:
            t = srv.submit(ds[owners[tf]], tf_ids[tf], w, h, cam[0], cam[1], spv)
            img, res = srv.wait(t)
            assert res["batch_size"] == 1
            alone.append(img)
    for i in range(12):
        assert np.array_equal(alone[i], mixed[i][0]), i
    assert {tf for tf, *_ in reqs} == set(range(len(tfs)))
    # the renderer API draws the same pixels
    for i, (tf, w, h, cam, spv) in enumerate(reqs[:14]):
        m, t, kw = tfs[tf]
        with Renderer() as r:
            r.loadVolume(hosts[owners[tf]], brick_size=64, overlap=2)
            r.resize((w, h))
            r.setRenderMode(m)
            if m in (GBVR_RM_1DTRANS, GBVR_RM_MIP):
                r.set1DTrans(t)
            elif m == GBVR_RM_2DTRANS:
                r.set2DTrans(t, kw["grad_max"])
            else:
                r.setIsoValue(kw["iso"], kw["iso_rgb"])
            r.setSampleRateModifier(spv)
            r.setView(*cam)
            r.paint()
            assert np.array_equal(r.readFramebuffer(0), mixed[i][0]), i
    assert any(img[..., 3].max() > 0 for img, _ in mixed)


def test_admission_limits(setup):
    vols, _, tfs, owners = setup
    with Server(max_batch=4, fb_budget_bytes=2 * 64 * 64 * 4, slots=2) as srv:
        d = srv.add_synthetic(vols[0], brick_size=64, overlap=2)
        t = srv.add_tf(d, tfs[0][0], tfs[0][1])
        cam = orbit_camera(10.0, 10.0, 2.5 * workloads.DIAG, 45.0, 64, 64)
        # fits one slot exactly: admitted, one request per batch
        ok = [srv.submit(d, t, 64, 64, *cam) for _ in range(3)]
        assert all(srv.wait(k)[1]["batch_size"] == 1 for k in ok)
        # larger than a slot's framebuffer share: never admissible, rejected at submit
        with pytest.raises(GbvrError) as e:
            srv.submit(d, t, 65, 64, *orbit_camera(10.0, 10.0, 4.0, 45.0, 65, 64))
        assert e.value.code == -1
        with pytest.raises(GbvrError):
            srv.submit(d, t + 5, 64, 64, *cam)


def _serve(setup, reqs, **params):
    """Render `reqs` as one burst on a new server; (images, stats, server tune)."""
    vols, _, tfs, owners = setup
    do_tune = params.pop("_tune", False)
    with Server(**params) as srv:
        ds = [srv.add_synthetic(v, brick_size=64, overlap=2) for v in vols]
        tf_ids = [srv.add_tf(ds[owners[i]], m, t, **kw) for i, (m, t, kw) in enumerate(tfs)]
        tune = srv.autotune(96, 96, 6) if do_tune else None
        tickets = [srv.submit(ds[owners[tf]], tf_ids[tf], w, h, cam[0], cam[1], spv) for tf, w, h, cam, spv in reqs]
        imgs = [srv.wait(t)[0] for t in tickets]
        return imgs, srv.stats(), tune


def _big_requests(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        tf = int(rng.integers(0, 6))
        w, h = [(480, 320), (640, 480), (320, 320)][int(rng.integers(0, 3))]
        cam = orbit_camera(float(rng.uniform(0, 360)), float(rng.uniform(-40, 40)),
                           float(rng.uniform(1.3, 2.0)) * workloads.DIAG, 45.0, w, h)
        out.append((tf, w, h, cam, 1.5))
    return out


def test_batches_overlap_on_the_device_and_images_do_not_change(setup):
    """Three slots on three streams: consecutive batches' kernel spans overlap
    (the later batch starts before the earlier ends); the images equal those
    of a one-slot server bit for bit."""
    reqs = _big_requests(60, 21)
    multi, st, _ = _serve(setup, reqs, max_batch=6, fb_budget_bytes=64 << 20, slots=3)
    single, st1, _ = _serve(setup, reqs, max_batch=6, fb_budget_bytes=64 << 20, slots=1)
    for a, b in zip(multi, single):
        assert np.array_equal(a, b)
    assert st["completed"] == len(reqs) and st["batches"] >= 10
    assert st["overlap_checked"] >= 5 and st["overlapped"] >= 1, st
    assert st1["overlapped"] == 0  # one stream: batches run one after the other


def test_memory_budget_evicts_and_uploads(setup):
    """A brick-pool budget that holds one dataset at a time: requests over all
    three datasets are served by evicting and re-uploading pools, with the
    same images as a server without a budget."""
    reqs = _requests(40, 31)
    free, st_free, _ = _serve(setup, reqs, max_batch=8, fb_budget_bytes=8 << 20)
    assert st_free["evictions"] == 0 and st_free["uploads"] == 0
    # pool sizes from an unbudgeted server's resident bytes
    vols, _, tfs, owners = setup
    sizes = []
    with Server() as srv:
        prev = 0
        for v in vols:
            srv.add_synthetic(v, brick_size=64, overlap=2)
            cur = srv.stats()["resident_bytes"]
            sizes.append(cur - prev)
            prev = cur
    budget = max(sizes) + 1
    tight, st, _ = _serve(setup, reqs, max_batch=8, fb_budget_bytes=8 << 20, device_pool_bytes=budget)
    for a, b in zip(tight, free):
        assert np.array_equal(a, b)
    assert st["evictions"] >= 2 and st["uploads"] >= 3 and st["resident_bytes"] <= budget, st
    # a pool above the budget can never be admitted: rejected when added
    with Server(device_pool_bytes=min(sizes) - 1) as srv:
        with pytest.raises(GbvrError) as e:
            srv.add_synthetic(vols[int(np.argmax(sizes))], brick_size=64, overlap=2)
        assert e.value.code == -1 and "device_pool_bytes" in str(e.value)


def test_autotuned_shapes_keep_the_images(setup):
    reqs = _requests(30, 41)
    base, _, _ = _serve(setup, reqs, max_batch=8, fb_budget_bytes=8 << 20)
    tuned, st, tune = _serve(setup, reqs, max_batch=8, fb_budget_bytes=8 << 20, _tune=True)
    for a, b in zip(tuned, base):
        assert np.array_equal(a, b)
    groups = {(t["dtype"], t["mode"]) for t in tune}
    # u8 1D and MIP, u16 1D, 2D and isosurface, f32 1D
    assert groups == {(0, 0), (0, 3), (1, 0), (1, 1), (1, 2), (2, 0)}, groups
    for t in tune:
        assert t["tile_w"] in (4, 8, 16) and t["ctas_per_sm"] >= 1 and t["candidates"] >= 9
        assert 0 < t["best_ms"] <= t["default_ms"]


def test_wait_timeout_keeps_the_ticket(setup):
    vols, _, tfs, owners = setup
    with Server(max_batch=64, fb_budget_bytes=512 << 20) as srv:
        d = srv.add_synthetic(vols[1], brick_size=64, overlap=2)
        t = srv.add_tf(d, tfs[1][0], tfs[1][1])
        cams = [orbit_camera(5.0 * i, 10.0, 1.3 * workloads.DIAG, 45.0, 1920, 1080) for i in range(32)]
        tickets = [srv.submit(d, t, 1920, 1080, *c) for c in cams]
        # the last request cannot be done 10 microseconds after a burst of 32 full-HD frames
        with pytest.raises(GbvrError) as e:
            srv.wait(tickets[-1], timeout_s=1e-5)
        assert e.value.code == -9
        # the ticket is still valid: waiting without a limit returns the image
        img, res = srv.wait(tickets[-1])
        assert res["status"] == 0 and img.shape == (1080, 1920, 4)
        for k in tickets[:-1]:
            srv.wait(k)


def test_failed_launch_fails_its_batch_and_the_worker_goes_on(setup, monkeypatch):
    """A batch launch that throws (host-side failure injection) fails that
    batch's requests with a status; the next batch renders normally."""
    vols, _, tfs, owners = setup
    with Server(max_batch=4, fb_budget_bytes=8 << 20) as srv:
        d = srv.add_synthetic(vols[0], brick_size=64, overlap=2)
        t = srv.add_tf(d, tfs[0][0], tfs[0][1])
        cam = orbit_camera(30.0, 10.0, 2.0 * workloads.DIAG, 45.0, 64, 64)
        monkeypatch.setenv("GBVR_FAULT_INJECT", "server_launch")
        bad = srv.submit(d, t, 64, 64, *cam)
        with pytest.raises(GbvrError) as e:
            srv.wait(bad)
        assert e.value.code == -1 and "injected" in str(e.value)
        monkeypatch.delenv("GBVR_FAULT_INJECT")
        good = srv.submit(d, t, 64, 64, *cam)
        img, res = srv.wait(good)
        assert res["status"] == 0 and img[..., 3].max() > 0
