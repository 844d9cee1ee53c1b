"""Batched forward (one pipeline pass over views of several scenes and
resolutions, captured and replayed as a CUDA graph) against the
single-view forward of each view.

Bars: the batch's key count equals the sum of the views' counts (integer,
exact); every image within max-abs 2/255 and PSNR >= 50 dB of its
single-view render (keys of equal tile and depth may blend in another
order); the graph replay with new cameras matches fresh single-view renders.
"""
import pytest
import torch

from polysplat_gb300 import Camera, Rasterizer, Scene, scenes
from polysplat_gb300 import _lib as R
from polysplat_gb300._lib import GsrError
from polysplat_gb300.batch import Batcher, View

from helpers import image_stats

pytestmark = pytest.mark.gpu

E2E = "preranges_smem_persistent_lite_e2e"


def _scenes(dev):
    raws = [scenes.subsample(scenes.scene_clustered(600_000, seed=1), 60_000, seed=2),
            scenes.scene_clustered(50_000, seed=33),
            scenes.subsample(scenes.scene_plain_small(), 30_000, seed=1)]
    return [Scene.from_raw(r, dev) for r in raws]


def _cams(az):
    f = scenes.focal_for
    return [(0, Camera.from_spec(scenes.camera_front(640, 360, 1400.0 / 3))),
            (1, Camera.from_spec(scenes.orbit_camera(8.0, 0.7 + az, 0.3, 1280, 720, f(1280)))),
            (2, Camera.from_spec(scenes.camera_front(800, 600, 600.0))),
            (1, Camera.from_spec(scenes.orbit_camera(9.0, 2.0 + az, -0.2, 320, 240, f(320)))),
            (0, Camera.from_spec(scenes.orbit_camera(10.0, 1.0 + az, 0.1, 1920, 1080, f(1920))))]


def _single(scs, views, bg):
    outs, total = [], 0
    for si, cam in views:
        r = Rasterizer(scs[si], 4_000_000, 1 << 16)
        img, st = r.forward(scs[si], cam, bg, render_variant=E2E, return_stats=True)
        outs.append(img.clone())
        total += st["num_rendered"]
    return outs, total


def test_batch_matches_single_view_and_replays(cuda_device):
    scs = _scenes(cuda_device)
    bg = torch.tensor([0.1, 0.2, 0.3])
    b = Batcher(8, 8_000_000, sum(s.num_vertex for s in scs) * 2, 40_000, cuda_device)
    stream = torch.cuda.Stream(cuda_device)
    for rep, az in enumerate([0.0, 0.0, 0.0, 0.4]):  # eager, captured, replayed, replayed with new cameras
        views = _cams(az)
        ref, total = _single(scs, views, bg)
        torch.cuda.synchronize()
        vs = [View(si, cam, bg) for si, cam in views]
        with torch.cuda.stream(stream):
            b.render(scs, vs, variant=R.RENDER_PERSISTENT_FUSED, half=True, use_graph=True, stream=stream)
        m = b.finish(stream)
        assert m == total, (rep, m, total)
        for (si, cam), v, r in zip(views, vs, ref):
            s = image_stats(v.out.cpu().numpy(), r.cpu().numpy())
            assert s["max_abs"] <= 2 and s["psnr"] >= 50.0, (rep, cam.width, s)
    assert b.graphs == 1  # one batch shape: captured once, replayed after
    b.close()


def test_batch_reports_overflow(cuda_device):
    scs = _scenes(cuda_device)
    b = Batcher(4, 10_000, sum(s.num_vertex for s in scs), 40_000, cuda_device)
    views = [View(si, cam) for si, cam in _cams(0.0)[:3]]
    b.render(scs, views, use_graph=False)
    with pytest.raises(GsrError) as ei:
        b.finish()
    assert ei.value.status == R.GSR_OVERFLOW and ei.value.num > 10_000
    b.close()


def test_batch_rejects_bad_layouts(cuda_device):
    scs = _scenes(cuda_device)
    b = Batcher(2, 100_000, 100_000, 1000, cuda_device)
    views = [View(si, cam) for si, cam in _cams(0.0)[:3]]
    with pytest.raises(GsrError):
        b.render(scs, views)  # more views than max_views
    with pytest.raises(GsrError):
        b.render(scs, views[:2])  # more Gaussians / tiles than the batcher holds
    b.close()


def test_new_batcher_first_batch_on_a_nonblocking_stream(cuda_device):
    """A batcher zero-fills its buffer block when it is created.  A batch
    launched at once on a fresh non-blocking stream (which does not wait for
    the legacy default stream the fill runs on) must find the fill finished:
    creation waits for it.  Each round builds a large block (2^26 keys, a fill
    of a few milliseconds) and renders on a new stream straight away."""
    scs = _scenes(cuda_device)
    bg = torch.tensor([0.0, 0.0, 0.0])
    views = _cams(0.0)[:3]
    ref, total = _single(scs, views, bg)
    torch.cuda.synchronize()
    for _ in range(3):
        b = Batcher(4, 1 << 26, sum(s.num_vertex for s in scs), 1 << 16, cuda_device)
        stream = torch.cuda.Stream(cuda_device)
        vs = [View(si, cam, bg) for si, cam in views]
        with torch.cuda.stream(stream):
            b.render(scs, vs, variant=R.RENDER_PERSISTENT_FUSED, half=True, use_graph=False, stream=stream)
        assert b.finish(stream) == total
        for v, r in zip(vs, ref):
            s = image_stats(v.out.cpu().numpy(), r.cpu().numpy())
            assert s["max_abs"] <= 2 and s["psnr"] >= 50.0, s
        b.close()
