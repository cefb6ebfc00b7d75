"""Asynchronous batches: a pipeline of steps over two framebuffer sets, the
read-back of one step overlapping the render of the next, gives every step
the images of a synchronous batch of the same views."""
import numpy as np
import pytest
import torch

from imagevis3d_gb300 import GbvrError, Renderer, synth_params, workloads

pytestmark = pytest.mark.gpu

W, H = 96, 72


@pytest.fixture(scope="module")
def sp():
    return synth_params((80, 70, 60), np.uint8, 23, 8, (3.0, 9.0), (0.3, 1.0), 255.0, noise_kind=1, noise_amp=4.0,
                        vmax=255.0)


def _renderer(sp):
    r = Renderer()
    r.loadSynthetic(sp, brick_size=32, overlap=2)
    r.resize((W, H))
    r.set1DTrans(workloads.tf1d_seeded(256, 23, 30.0, 255.0))
    r.setValueRange(0.0, 255.0)
    return r


def test_pipeline_steps_equal_synchronous_batches(sp):
    steps = [workloads.orbit_views(6, W, H, elevation=e, start=s) for e, s in
             ((10, 0), (30, 15), (-20, 40), (45, 70), (0, 100))]
    with _renderer(sp) as r:
        want = []
        for views in steps:
            r.paintBatch(views)
            want.append(r.readFramebuffers(0, len(views)).copy())
        host = [torch.empty((6, H, W, 4), dtype=torch.uint8).pin_memory() for _ in range(2)]
        for i, views in enumerate(steps):
            r.paintBatchAsync(views, i % 2)
            if i > 0:
                # host buffer i % 2 is rewritten every other step: in order on the read stream
                r.readFramebuffersAsync((i - 1) % 2, host[(i - 1) % 2])
        r.readFramebuffersAsync((len(steps) - 1) % 2, host[(len(steps) - 1) % 2])
        r.waitAsync()
        # the two host buffers hold the last two steps
        assert np.array_equal(host[(len(steps) - 1) % 2].numpy(), want[-1])
        assert np.array_equal(host[(len(steps) - 2) % 2].numpy(), want[-2])


def test_every_step_read_back_in_a_pipeline(sp):
    steps = [workloads.orbit_views(4, W, H, elevation=e, start=s) for e, s in ((5, 0), (25, 30), (-35, 60), (15, 90))]
    with _renderer(sp) as r:
        want = []
        for views in steps:
            r.paintBatch(views)
            want.append(r.readFramebuffers(0, len(views)).copy())
        outs = [torch.empty((4, H, W, 4), dtype=torch.uint8).pin_memory() for _ in steps]
        for i, views in enumerate(steps):
            r.paintBatchAsync(views, i % 2)
            if i > 0:
                r.readFramebuffersAsync((i - 1) % 2, outs[i - 1])
        r.readFramebuffersAsync((len(steps) - 1) % 2, outs[-1])
        r.waitAsync()
        for i in range(len(steps)):
            assert np.array_equal(outs[i].numpy(), want[i]), i
        # a synchronous call afterwards sees its own frames
        r.paintBatch(steps[0])
        assert np.array_equal(r.readFramebuffers(0, 4), want[0])


def test_consumer_waits_for_one_read_back(sp):
    """A consumer takes step i - 1's frames from host memory while step i
    renders: waiting for that slot's read-back is enough."""
    steps = [workloads.orbit_views(3, W, H, elevation=e, start=s) for e, s in
             ((0, 0), (20, 25), (-15, 50), (35, 75), (10, 110), (-40, 140))]
    with _renderer(sp) as r:
        want = []
        for views in steps:
            r.paintBatch(views)
            want.append(r.readFramebuffers(0, len(views)).copy())
        host = [torch.empty((3, H, W, 4), dtype=torch.uint8).pin_memory() for _ in range(2)]
        got = []
        for i, views in enumerate(steps):
            r.paintBatchAsync(views, i % 2)
            if i > 0:
                r.readFramebuffersAsync((i - 1) % 2, host[(i - 1) % 2])
                r.waitRead((i - 1) % 2)
                got.append(host[(i - 1) % 2].numpy().copy())
        r.readFramebuffersAsync((len(steps) - 1) % 2, host[(len(steps) - 1) % 2])
        r.waitRead((len(steps) - 1) % 2)
        got.append(host[(len(steps) - 1) % 2].numpy().copy())
        r.waitAsync()
        for i in range(len(steps)):
            assert np.array_equal(got[i], want[i]), i


def test_async_errors(sp):
    with _renderer(sp) as r:
        with pytest.raises(GbvrError):
            r.readFramebuffersAsync(1, np.zeros((1, H, W, 4), np.uint8))  # nothing rendered into slot 1
        views = workloads.orbit_views(2, W, H)
        with pytest.raises(GbvrError):
            r.paintBatchAsync(views, 2)
        with pytest.raises(GbvrError):
            r.waitRead(-1)
        r.waitRead(0)  # nothing queued: returns at once
        r.paintBatchAsync(views, 1)
        with pytest.raises(GbvrError):
            r.readFramebuffersAsync(1, np.zeros((1, H, W, 4), np.uint8), 0, 2)  # too small
        r.waitAsync()


def test_async_batches_after_a_captured_path(sp):
    """A captured path first (it creates the read stream), then asynchronous
    batches of 5 views (the read-back split unevenly over two copy streams) on
    the same renderer: every step equals its synchronous batch."""
    steps = [workloads.orbit_views(5, W, H, elevation=e, start=s) for e, s in ((12, 5), (-18, 50), (33, 95))]
    with _renderer(sp) as r:
        want = []
        for views in steps:
            r.paintBatch(views)
            want.append(r.readFramebuffers(0, len(views)).copy())
        cap = torch.empty((5, H, W, 4), dtype=torch.uint8).pin_memory()
        r.paintPath(steps[0], capture=cap)
        outs = [torch.empty((5, H, W, 4), dtype=torch.uint8).pin_memory() for _ in steps]
        for i, views in enumerate(steps):
            r.paintBatchAsync(views, i % 2)
            r.readFramebuffersAsync(i % 2, outs[i])
        r.waitAsync()
        for o, w in zip(outs, want):
            assert np.array_equal(o.numpy(), w)
