"""Serving: every request's image from the mixed, continuously batched run
equals its image rendered alone (within max-abs 2/255 and PSNR >= 50 dB),
through both lanes; the real-time replay completes every request; the
autotuner returns a configuration that serves."""

import numpy as np
import pytest
import torch

from polysplat_gb300 import Camera, Rasterizer, Scene, scenes
from polysplat_gb300.serving import PlainServer, Server, TuneConfig, autotune

from helpers import image_stats

pytestmark = pytest.mark.gpu

RES = [(320, 240), (640, 360), (800, 600), (1280, 720)]


def _mix(n, rate_hz, seed=7):
    rng = np.random.default_rng(seed)
    raws = [scenes.scene_clustered(40_000, seed=11), scenes.scene_clustered(120_000, seed=12),
            scenes.scene_clustered(250_000, seed=13)]
    reqs, t = [], 0.0
    for k in range(n):
        t += rng.exponential(1.0 / rate_hz)
        w, h = RES[int(rng.integers(0, len(RES)))]
        cam = scenes.orbit_camera(rng.uniform(6, 12), rng.uniform(0, 6.28), rng.uniform(-0.5, 0.5), w, h,
                                  scenes.focal_for(w), id=k)
        reqs.append(scenes.Request(t, int(rng.integers(0, len(raws))), cam))
    return raws, reqs


@pytest.mark.parametrize("quad", [False, True], ids=["tile_keys", "quad_keys"])
def test_served_images_equal_alone(cuda_device, quad):
    """Both key layouts the autotuner considers for the batched lane: each
    request against the single-view 16x16 E2E forward."""
    raws, reqs = _mix(40, 1000.0)
    scs = [Scene.from_raw(r, cuda_device) for r in raws]
    # both lanes take work: a quad key stands for about 2.5 per-tile keys, so
    # the large-lane threshold scales with the layout's key estimate
    cfg = TuneConfig(max_views=6, large_keys=160_000 if quad else 400_000, quad=quad)
    srv = Server(scs, cuda_device, budget_bytes=6 << 30, config=cfg)
    st = srv.run(reqs, realtime=False)
    torch.cuda.synchronize()
    assert st.requests == len(reqs) and st.large > 0 and st.batches > 0 and st.mean_batch > 1.0
    alone = Rasterizer(max(scs, key=lambda s: s.num_vertex), 8_000_000, 1 << 16)
    for r in reqs:
        img = alone.forward(scs[r.scene], Camera.from_spec(r.camera), torch.zeros(3),
                            render_variant="preranges_smem_persistent_lite_e2e")
        s = image_stats(r.out.cpu().numpy(), img.cpu().numpy())
        assert s["max_abs"] <= 2 and s["psnr"] >= 50.0, (r.scene, r.camera.width, s)
    srv.close()


def test_realtime_replay_and_plain_baseline(cuda_device):
    raws, reqs = _mix(30, 600.0, seed=8)
    scs = [Scene.from_raw(r, cuda_device) for r in raws]
    srv = Server(scs, cuda_device, budget_bytes=6 << 30, config=TuneConfig(max_views=4, large_keys=600_000))
    st = srv.run(reqs, realtime=True)
    assert st.requests == 30 and all(r.latency_s > 0 for r in reqs) and st.p99_ms >= st.p50_ms
    srv.close()
    plain = PlainServer(scs, 8_000_000, cuda_device)
    pst, _ = plain.run(reqs, realtime=True)
    assert pst.requests == 30 and pst.p50_ms > 0


def test_autotune_returns_a_serving_config(cuda_device):
    raws, reqs = _mix(16, 1000.0, seed=9)
    scs = [Scene.from_raw(r, cuda_device) for r in raws]
    best, table = autotune(scs, reqs, cuda_device, budget_bytes=6 << 30,
                           axes=[("max_views", [2]), ("large_keys", [300_000])])
    assert len(table) >= 3 and isinstance(best, TuneConfig)
    srv = Server(scs, cuda_device, budget_bytes=6 << 30, config=best)
    assert srv.run(reqs, realtime=False).requests == 16
    srv.close()


def test_large_lane_frame_beyond_its_buffers_fails_alone(cuda_device):
    """Every request takes the large lane, whose key buffers are capped at
    the median frame's key count: the bigger frames fail on their own request
    with the true key count, and every other request is served with its
    correct image."""
    raws, reqs = _mix(16, 1000.0, seed=10)
    scs = [Scene.from_raw(r, cuda_device) for r in raws]
    alone = Rasterizer(max(scs, key=lambda s: s.num_vertex), 8_000_000, 1 << 16)
    want = []
    for r in reqs:
        img, stt = alone.forward(scs[r.scene], Camera.from_spec(r.camera), torch.zeros(3),
                                 render_variant="preranges_smem_persistent_lite_e2e", return_stats=True)
        want.append((img.clone(), int(stt["num_rendered"])))
    cap = int(np.median([n for _, n in want]))
    srv = Server(scs, cuda_device, budget_bytes=6 << 30, config=TuneConfig(max_views=4, large_keys=0),
                 large_capacity=cap)
    st = srv.run(reqs, realtime=False)
    torch.cuda.synchronize()
    n_fail = 0
    for r, (img, n) in zip(reqs, want):
        if n > cap:
            n_fail += 1
            assert r.error is not None and r.error.status == 1 and r.error.num == n, (n, cap, r.error)
            assert r.out is None and r.latency_s is None
        else:
            assert r.error is None
            s = image_stats(r.out.cpu().numpy(), img.cpu().numpy())
            assert s["max_abs"] <= 2 and s["psnr"] >= 50.0, (r.scene, r.camera.width, s)
    assert 0 < n_fail < len(reqs) and st.failed == n_fail and st.requests == len(reqs) - n_fail
    srv.close()
