"""GPU parity of the ES ("early sorting") operators called one by one in the
reference's order (example.py:495-580): pass A, depth sort + scan, pass B,
tile sort, then tile ranges and the persistent render.

Bars (integer work bit-exact):
* pass A: counts sum to the single-pass pair count; culled Gaussians carry
  count 0 and depth FLT_MAX; features equal the single-pass features;
* depth sort + scan: perm is the stable sort of depth_natural, the gathered
  counts, their exclusive scan and the device total exact;
* pass B + tile sort: the sorted (tile, Gaussian) sequence equals the
  depth-first forward's bit for bit, every pair's tile lies inside its
  Gaussian's packed rectangle, and the 64-bit keys are tile << 32;
* image: equal to the depth-first forward's, within max-abs 2/255 and PSNR
  >= 50 dB of the single-pass forward's.
"""
import numpy as np
import pytest
import torch

from polysplat_gb300 import Camera, Scene, ops
from polysplat_gb300 import _lib as R
from polysplat_gb300._lib import GsrError

from helpers import image_stats
from test_gpu_depth_first import CASES, _depth_first, _single_pass

pytestmark = pytest.mark.gpu

FLT_MAX_BITS = 0x7F7FFFFF


class _Es:
    """The reference rasterizer's ES buffers (example.py:87-107)."""

    def __init__(self, P, W, H, cap, dev):
        i32, f32 = torch.int32, torch.float32
        self.tiles_per_gauss = torch.zeros(P, device=dev, dtype=i32)
        self.conic_power_raw = torch.zeros((P, 4), device=dev, dtype=f32)
        self.depth_natural = torch.zeros(P, device=dev, dtype=f32)
        self.rect_bounds = torch.zeros((P, 2), device=dev, dtype=i32)
        self.identity = torch.zeros(P, device=dev, dtype=i32)
        self.perm = torch.zeros(P, device=dev, dtype=i32)
        self.depth_sorted = torch.zeros(P, device=dev, dtype=f32)
        self.tiles_sorted = torch.zeros(P, device=dev, dtype=i32)
        self.cum = torch.zeros(P, device=dev, dtype=i32)
        self.total = torch.zeros(1, device=dev, dtype=i32)
        self.tku = torch.zeros(cap, device=dev, dtype=i32)
        self.tks = torch.zeros(cap, device=dev, dtype=i32)
        self.vu = torch.zeros(cap, device=dev, dtype=i32)
        self.vs = torch.zeros(cap, device=dev, dtype=i32)
        self.ks = torch.zeros(cap, device=dev, dtype=torch.int64)
        self.scan = torch.zeros(ops.get_es_scan_buffer_size(P), device=dev, dtype=torch.int8)
        self.ws = torch.zeros(ops.get_sort_buffer_size(max(cap, P)), device=dev, dtype=torch.int8)
        self.xy = torch.zeros((P, 2), device=dev, dtype=f32)
        self.rgbd = torch.zeros((P, 4), device=dev, dtype=f32)
        self.con = torch.zeros((P, 4), device=dev, dtype=f32)
        tiles = ((W + 15) // 16) * ((H + 15) // 16)
        self.ranges = torch.zeros((tiles, 2), device=dev, dtype=i32)
        self.out = torch.zeros((H, W, 3), device=dev, dtype=torch.uint8)


def _es_chain(scene, c, half, cap, dev, bg):
    P = scene.num_vertex
    e = _Es(P, c.width, c.height, cap, dev)
    pass_a = ops.preprocess_es_pass_a_half_sh if half else ops.preprocess_es_pass_a
    pass_a(scene.position, scene.shs_half if half else scene.shs, scene.opacity, scene.cov3d, c.width, c.height,
           16, 16, c.position, c.rotation, c.focal_x, c.focal_y, c.zFar, c.zNear, e.xy, e.rgbd, e.con,
           e.tiles_per_gauss, e.conic_power_raw, e.depth_natural, e.rect_bounds)
    ops.es_depth_sort_and_scan(P, e.tiles_per_gauss, e.depth_natural, e.identity, e.perm, e.depth_sorted,
                               e.tiles_sorted, e.cum, e.total, e.ws, e.scan)
    ops.preprocess_es_pass_b(P, c.width, c.height, 16, 16, e.perm, e.cum, e.tiles_sorted, e.xy, e.conic_power_raw,
                             e.rect_bounds, e.tku, e.vu)
    m = int(e.total.cpu()[0])
    ops.es_tile_sort(m, c.width, c.height, 16, 16, e.tku, e.vu, e.tks, e.vs, e.ks, e.ws)
    ops.precompute_tile_ranges(m, c.width, c.height, 16, 16, e.ks, e.ranges)
    ops.render_16x16_preranges_smem_persistent_lite(m, c.width, c.height, e.xy, e.rgbd, e.con, e.vs, e.ranges, bg,
                                                     e.out)
    torch.cuda.synchronize()
    return m, e


@pytest.mark.parametrize("case,half", [(k, True) for k in CASES] + [("orbit_1280x720", False)])
def test_es_ops_match_depth_first_and_single_pass(cuda_device, case, half):
    raw, cam = CASES[case][0](), CASES[case][1]()
    scene = Scene.from_raw(raw, cuda_device)
    c = Camera.from_spec(cam)
    bg = torch.tensor([0.1, 0.3, 0.7])
    cap = 8_000_000
    P = scene.num_vertex
    m1, a = _single_pass(scene, c, half, cap, cuda_device, bg)
    m2, d = _depth_first(scene, c, half, cap, cuda_device, bg)
    m, e = _es_chain(scene, c, half, cap, cuda_device, bg)
    assert m == m1 == m2

    # pass A
    cnt = e.tiles_per_gauss.cpu().numpy().astype(np.int64)
    dbits = e.depth_natural.cpu().numpy().view(np.uint32)
    assert cnt.sum() == m and (cnt >= 0).all()
    assert (cnt[dbits == FLT_MAX_BITS] == 0).all()
    hit = cnt > 0
    for name in ("xy", "rgbd", "con"):
        mine, ref = getattr(e, name).cpu().numpy()[hit], getattr(a, name).cpu().numpy()[hit]
        assert np.array_equal(mine.view(np.uint32), ref.view(np.uint32)), name
    cpr = e.conic_power_raw.cpu().numpy()[hit]
    con = e.con.cpu().numpy()[hit]
    np.testing.assert_allclose(cpr[:, 0] * np.float32(-0.5 / np.log(2.0)), con[:, 0], rtol=1e-6, atol=0)

    # depth sort + scan
    ref_perm = torch.sort(e.depth_natural, stable=True).indices.cpu().numpy()
    perm = e.perm.cpu().numpy().astype(np.int64)
    assert np.array_equal(perm, ref_perm)
    assert np.array_equal(e.identity.cpu().numpy(), np.arange(P))
    assert np.array_equal(e.depth_sorted.cpu().numpy().view(np.uint32), dbits[perm])
    ts = e.tiles_sorted.cpu().numpy().astype(np.int64)
    assert np.array_equal(ts, cnt[perm])
    cum = e.cum.cpu().numpy().astype(np.int64)
    assert np.array_equal(cum, np.concatenate([[0], np.cumsum(ts)[:-1]]))

    # pass B + tile sort against the depth-first forward
    tks = e.tks.cpu().numpy()[:m]
    vs = e.vs.cpu().numpy()[:m]
    assert np.array_equal(tks, d.ks.cpu().numpy()[:m])
    assert np.array_equal(vs, d.vs.cpu().numpy()[:m])
    assert np.array_equal(e.ks.cpu().numpy()[:m], tks.astype(np.int64) << 32)
    assert np.array_equal(e.ranges.cpu().numpy(), d.ranges.cpu().numpy())
    rb = e.rect_bounds.cpu().numpy().astype(np.int64)[vs]
    gx = (c.width + 15) // 16
    tx, ty = tks.astype(np.int64) % gx, tks.astype(np.int64) // gx
    x0, y0 = rb[:, 0] & 0xFFFF, (rb[:, 0] >> 16) & 0xFFFF
    x1, y1 = rb[:, 1] & 0xFFFF, (rb[:, 1] >> 16) & 0xFFFF
    assert ((tx >= x0) & (tx < x1) & (ty >= y0) & (ty < y1)).all()

    # images
    assert np.array_equal(e.out.cpu().numpy(), d.out.cpu().numpy())
    s = image_stats(e.out.cpu().numpy(), a.out.cpu().numpy())
    assert s["max_abs"] <= 2 and s["psnr"] >= 50.0, s


@pytest.mark.parametrize("case,half", [(k, True) for k in CASES] + [("orbit_1280x720", False)])
def test_es_ops_vs_reference_es_kernels(cuda_device, case, half):
    """Every buffer of the ES steps against the reference's own ES kernels
    (preprocessCUDA_ES_PassA / PassB, preprocess.cu:692-1248) and its CUB
    depth sort, scan and tile sort (sort.cu:151-285), on the same inputs.
    All integer or copied data: bit-exact.  Within one tile every Gaussian
    contributes at most one pair, so the tile-sorted values are exact too."""
    from oracle import refkernels as RK

    if not RK.available():
        pytest.skip("reference kernels not built")
    raw, cam = CASES[case][0](), CASES[case][1]()
    scene = Scene.from_raw(raw, cuda_device)
    c = Camera.from_spec(cam)
    cap = 8_000_000
    m, e = _es_chain(scene, c, half, cap, cuda_device, torch.tensor([0.0, 0.0, 0.0]))
    r = RK.es_chain(scene, cam, half, cap)
    assert m == r["m"]
    u32 = lambda t: t.cpu().numpy().view(np.uint32)
    # pass A: counts and depths of every Gaussian; the records pass B reads
    # (conic + power, rectangle) and the features, for the Gaussians that
    # hit a tile (the reference leaves the other rows as they were)
    for name in ("tiles_per_gauss", "depth_natural"):
        assert np.array_equal(u32(getattr(e, name)), u32(r[name])), name
    hit = e.tiles_per_gauss.cpu().numpy() > 0
    for name in ("conic_power_raw", "rect_bounds", "xy", "rgbd", "con"):
        mine, ref = u32(getattr(e, name))[hit], u32(r[name])[hit]
        assert np.array_equal(mine, ref), (name, int((mine != ref).any(axis=-1).sum()))
    # depth sort + scan
    for name in ("identity", "perm", "depth_sorted", "tiles_sorted", "cum", "total"):
        assert np.array_equal(u32(getattr(e, name)), u32(r[name])), name
    # pass B: each Gaussian's pairs fill its range [cum[s], cum[s] + count[s])
    tku, vu = u32(e.tku)[:m], u32(e.vu)[:m]
    rtku, rvu = u32(r["tku"])[:m], u32(r["vu"])[:m]
    assert np.array_equal(vu, rvu)  # the range owner's index at every position
    own = np.repeat(np.arange(scene.num_vertex), e.tiles_sorted.cpu().numpy())
    assert np.array_equal(tku[np.lexsort((tku, own))], rtku[np.lexsort((rtku, own))])
    # tile sort and the rebuilt 64-bit keys
    assert np.array_equal(u32(e.tks)[:m], u32(r["tks"])[:m])
    assert np.array_equal(u32(e.vs)[:m], u32(r["vs"])[:m])
    assert np.array_equal(e.ks.cpu().numpy()[:m], r["ks"].cpu().numpy()[:m])


def test_es_pass_b_bounded_by_capacity(cuda_device):
    raw, cam = CASES["orbit_1280x720"][0](), CASES["orbit_1280x720"][1]()
    scene = Scene.from_raw(raw, cuda_device)
    c = Camera.from_spec(cam)
    bg = torch.tensor([0.0, 0.0, 0.0])
    m, e = _es_chain(scene, c, True, 4_000_000, cuda_device, bg)
    half = m // 2
    guard = 4096
    tku = torch.full((half + guard,), -7, device=cuda_device, dtype=torch.int32)
    vu = torch.full((half + guard,), -7, device=cuda_device, dtype=torch.int32)
    ops.preprocess_es_pass_b(scene.num_vertex, c.width, c.height, 16, 16, e.perm, e.cum, e.tiles_sorted, e.xy,
                             e.conic_power_raw, e.rect_bounds, tku[:half], vu[:half])
    torch.cuda.synchronize()
    assert np.array_equal(tku[:half].cpu().numpy(), e.tku[:half].cpu().numpy())
    assert np.array_equal(vu[:half].cpu().numpy(), e.vu[:half].cpu().numpy())
    assert (tku[half:].cpu().numpy() == -7).all() and (vu[half:].cpu().numpy() == -7).all()
    with pytest.raises(GsrError) as ei:
        ops.es_tile_sort(m, c.width, c.height, 16, 16, tku[:half], vu[:half], e.tks, e.vs, e.ks, e.ws)
    assert ei.value.status == R.GSR_OVERFLOW


def test_es_empty_and_culled(cuda_device):
    raw, cam = CASES["small_800x600"][0](), CASES["small_800x600"][1]()
    scene = Scene.from_raw(raw, cuda_device)
    c = Camera.from_spec(cam)
    # camera moved far along its view direction: every Gaussian is behind it
    # (rotation columns are right, down, forward in world coordinates)
    away_pos = c.position + 1.0e4 * c.rotation[:, 2]
    e = _Es(scene.num_vertex, c.width, c.height, 1000, cuda_device)
    ops.preprocess_es_pass_a_half_sh(scene.position, scene.shs_half, scene.opacity, scene.cov3d, c.width, c.height,
                                     16, 16, away_pos, c.rotation, c.focal_x, c.focal_y, c.zFar, c.zNear, e.xy,
                                     e.rgbd, e.con, e.tiles_per_gauss, e.conic_power_raw, e.depth_natural,
                                     e.rect_bounds)
    ops.es_depth_sort_and_scan(scene.num_vertex, e.tiles_per_gauss, e.depth_natural, e.identity, e.perm,
                               e.depth_sorted, e.tiles_sorted, e.cum, e.total, e.ws, e.scan)
    torch.cuda.synchronize()
    assert int(e.total.cpu()[0]) == 0
    assert (e.depth_natural.cpu().numpy().view(np.uint32) == FLT_MAX_BITS).all()
    assert np.array_equal(e.perm.cpu().numpy(), np.arange(scene.num_vertex))
    ops.es_tile_sort(0, c.width, c.height, 16, 16, e.tku, e.vu, e.tks, e.vs, e.ks, e.ws)
    ops.es_depth_sort_and_scan(0, e.tiles_per_gauss, e.depth_natural, e.identity, e.perm, e.depth_sorted,
                               e.tiles_sorted, e.cum, e.total, e.ws, e.scan)
    torch.cuda.synchronize()
    assert int(e.total.cpu()[0]) == 0
