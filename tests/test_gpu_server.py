"""Serving loop: resident datasets and TF presets, requests from a burst and
one at a time; every image equals the same request rendered alone and the
same view rendered through the renderer API, bit for bit."""
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
    with Server(max_batch=4, fb_budget_bytes=2 * 64 * 64 * 4) as srv:
        d = srv.add_synthetic(vols[0], brick_size=64, overlap=2)
        t = srv.add_tf(d, tfs[0][0], tfs[0][1])
        cam = orbit_camera(10.0, 10.0, 2.5 * workloads.DIAG, 45.0, 64, 64)
        # fits one slot exactly: admitted, one request per batch
        ok = [srv.submit(d, t, 64, 64, *cam) for _ in range(3)]
        assert all(srv.wait(k)[1]["batch_size"] == 1 for k in ok)
        # larger than a slot: rejected, never rendered
        big = srv.submit(d, t, 65, 64, *orbit_camera(10.0, 10.0, 4.0, 45.0, 65, 64))
        with pytest.raises(GbvrError) as e:
            srv.wait(big)
        assert e.value.code == -1
        with pytest.raises(GbvrError):
            srv.submit(d, t + 5, 64, 64, *cam)
