"""Host-side logic of the server, on the CPU: how the small lane forms a
batch (arrival order, every budget respected, at least one request) and how
the key estimator learns from finished frames."""
import types

from polysplat_gb300.serving import KeyEstimator, Server, TuneConfig


def _req(scene, w, h, est):
    r = types.SimpleNamespace(scene=scene, est=est)
    r.cam = types.SimpleNamespace(width=w, height=h)
    return r


def _server(cfg, small_cap=10_000_000, max_g=100_000_000, tiles_cap=1 << 20, sizes=(1_000_000, 5_000_000)):
    return types.SimpleNamespace(cfg=cfg, small_cap=small_cap, max_g=max_g, tiles_cap=tiles_cap,
                                 scenes=[types.SimpleNamespace(num_vertex=n) for n in sizes])


def _take(srv, waiting):
    return Server._take_small(srv, waiting)


def test_batch_in_arrival_order_up_to_max_views():
    srv = _server(TuneConfig(max_views=3))
    waiting = [_req(0, 640, 360, 10_000) for _ in range(5)]
    first = list(waiting)
    got = _take(srv, waiting)
    assert got == first[:3] and waiting == first[3:]


def test_batch_stops_at_key_gaussian_and_tile_budgets():
    cfg = TuneConfig(max_views=8, block_x=16, block_y=16)
    # keys: each request is estimated at 1.25 x est
    srv = _server(cfg, small_cap=3_000_000)
    waiting = [_req(0, 640, 360, 1_000_000) for _ in range(4)]
    assert len(_take(srv, waiting)) == 2  # 2.5 M fits, 3.75 M does not
    # Gaussians of the views' scenes
    srv = _server(cfg, max_g=6_000_000)
    waiting = [_req(1, 640, 360, 10), _req(0, 640, 360, 10), _req(0, 640, 360, 10)]
    assert len(_take(srv, waiting)) == 2  # 5 M + 1 M
    # tiles: 1920x1080 at 16x16 is 120 x 68 = 8160 tiles
    srv = _server(cfg, tiles_cap=20_000)
    waiting = [_req(0, 1920, 1080, 10) for _ in range(3)]
    assert len(_take(srv, waiting)) == 2


def test_batch_tile_budget_knob():
    cfg = TuneConfig(max_views=8, block_x=32, block_y=32, max_batch_tiles=1 << 13)
    srv = _server(cfg)
    # 2160p at 32x32 is 120 x 68 = 8160 tiles: one such view per batch
    waiting = [_req(0, 3840, 2160, 10) for _ in range(3)]
    assert len(_take(srv, waiting)) == 1
    # 720p at 32x32 is 40 x 23 = 920 tiles: 8 fit (7360 tiles)
    waiting = [_req(0, 1280, 720, 10) for _ in range(10)]
    assert len(_take(srv, waiting)) == 8


def test_oversized_first_request_still_makes_a_batch():
    srv = _server(TuneConfig(max_views=4, max_batch_tiles=16), small_cap=10)
    waiting = [_req(0, 1920, 1080, 1_000_000), _req(0, 320, 240, 10)]
    got = _take(srv, waiting)
    assert len(got) == 1 and len(waiting) == 1


def test_key_estimator_learns_upwards_and_decays_slowly():
    scenes = [types.SimpleNamespace(num_vertex=2_000_000)]
    est = KeyEstimator(scenes)
    cam = types.SimpleNamespace(width=1000, height=1000)
    e0 = est(0, cam)
    assert e0 == int(2.5e-6 * 2_000_000 * 1_000_000) + 4096
    est.observe(0, cam, 9_000_000)  # 9 keys per pixel
    assert est(0, cam) == 9_000_000 + 4096
    est.observe(0, cam, 1_000_000)  # a lighter frame lowers the rate by 2 % only
    assert est(0, cam) == int(0.98 * 9.0 * 1_000_000) + 4096


def test_key_estimator_splits_a_batch_count_by_estimate():
    scenes = [types.SimpleNamespace(num_vertex=1_000_000), types.SimpleNamespace(num_vertex=3_000_000)]
    est = KeyEstimator(scenes)
    a, b = types.SimpleNamespace(width=100, height=100), types.SimpleNamespace(width=200, height=100)
    ea, eb = est(0, a), est(1, b)
    est.observe_batch([(0, a), (1, b)], 10 * (ea + eb))
    assert est(0, a) >= 9 * ea and est(1, b) >= 9 * eb


def test_quad_key_tiles():
    """With quad keys a view's key tile ids are its 2 x 2 groups of 16 x 16
    tiles: ceil(W / 32) x ceil(H / 32)."""
    cfg = TuneConfig(quad=True)
    assert cfg.key_tiles(1920, 1080) == 60 * 34
    assert cfg.key_tiles(3840, 2160) == 120 * 68
    assert cfg.key_tiles(1000, 584) == 32 * 19  # 63 x 37 tiles
    assert TuneConfig().key_tiles(1920, 1080) == 120 * 68
    assert cfg.batch_variant() & 0x100 and not TuneConfig().batch_variant() & 0x100

