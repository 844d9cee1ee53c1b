"""GPU parity against the reference's OWN CUDA kernels run on the same GB300.

The reference's preprocess / tile-range / render kernels are compiled from its
sources (oracle/ref_build.py) and launched by oracle/refrun.cpp with the same
camera matrices the library computes.  Bars:
  * sort and tile ranges fed the reference's preprocess output: bit-exact;
  * key lists: (tile, Gaussian) pair sets and depth bits compared; the
    number of differing pairs is asserted <= 1e-4 of M (fast-math boundary
    flips) and reported;
  * blend fed identical lists and features: max-abs <= 2/255, PSNR >= 50 dB
    (bit-exact expected; asserted separately where it holds);
  * whole frame: max-abs <= 2/255 and PSNR >= 50 dB.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from oracle import refkernels as RK
from polysplat_gb300 import Camera, Scene, ops, scenes

from helpers import compare_key_lists, image_stats

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not RK.available(), reason="reference device images not built")]

CASES = {
    "plain_100k_800x600": (lambda: scenes.scene_plain_small(), lambda: scenes.camera_front(800, 600, 600.0)),
    "clustered_300k_1280x720": (lambda: scenes.subsample(scenes.scene_clustered(3_000_000, seed=1), 300_000, seed=4),
                                lambda: scenes.camera_front(1280, 720, 1400.0 * 1280 / 1920)),
    "orbit_200k_1920x1080": (lambda: scenes.scene_clustered(200_000, seed=77),
                             lambda: scenes.orbit_camera(9.0, 2.1, -0.2, 1920, 1080, 1400.0)),
    "needles_50k_1920x1080": (lambda: scenes.scene_needles(50_000, seed=5),
                              lambda: scenes.orbit_camera(12.0, 0.4, 0.2, 1920, 1080, 1400.0)),
}

CAP = 8_000_000


def _bufs(dev, P):
    return dict(xy=torch.zeros((P, 2), device=dev), rgbd=torch.zeros((P, 4), device=dev),
                con=torch.zeros((P, 4), device=dev), cnt=torch.zeros(1, dtype=torch.int32, device=dev),
                keys=torch.zeros(CAP, dtype=torch.int64, device=dev),
                vals=torch.zeros(CAP, dtype=torch.int32, device=dev))


def _run_both(case, half, dev):
    raw, spec = CASES[case][0](), CASES[case][1]()
    scene = Scene.from_raw(raw, dev)
    cam = Camera.from_spec(spec)
    # this library first: its writes are clamped to the buffer and it reports
    # the true count; the reference's kernel writes unchecked, so it only runs
    # when the buffer is known to be far larger than the count
    ours = _bufs(dev, scene.num_vertex)
    fn = ops.preprocess_half_sh if half else ops.preprocess
    fn(scene.position, scene.shs_half if half else scene.shs, scene.opacity, scene.cov3d, cam.width, cam.height, 16,
       16, cam.position, cam.rotation, cam.focal_x, cam.focal_y, cam.zFar, cam.zNear, ours["xy"], ours["rgbd"],
       ours["con"], ours["keys"], ours["vals"], ours["cnt"])
    m = int(ours["cnt"].item())
    assert 2 * m < CAP, "case too large for the reference's unchecked key buffer"
    ref = _bufs(dev, scene.num_vertex)
    RK.preprocess(scene, spec, half, ref["xy"], scene.cov3d, ref["rgbd"], ref["con"], ref["cnt"], ref["keys"],
                  ref["vals"])
    torch.cuda.synchronize()
    assert int(ref["cnt"].item()) <= CAP
    return scene, spec, ref, ours


def _np(t, n, dt):
    return t[:n].cpu().numpy().view(dt)


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("half", [True, False])
def test_preprocess_keys_vs_reference(cuda_device, case, half):
    scene, spec, ref, ours = _run_both(case, half, cuda_device)
    mr, mo = int(ref["cnt"].item()), int(ours["cnt"].item())
    rk, rv = _np(ref["keys"], mr, np.uint64), _np(ref["vals"], mr, np.uint32)
    gk, gv = _np(ours["keys"], mo, np.uint64), _np(ours["vals"], mo, np.uint32)
    only_g, only_r, ulp = compare_key_lists(gk, gv, rk, rv)
    print("\n%s half=%s: M_ref=%d M_gsr=%d only_gsr=%d only_ref=%d depth_ulp=%d"
          % (case, half, mr, mo, only_g, only_r, ulp))
    assert only_g + only_r <= max(2, int(1e-4 * mr))
    assert ulp == 0
    # features of Gaussians both emitted
    em = np.intersect1d(np.unique(rv), np.unique(gv))
    for k in ("xy", "rgbd", "con"):
        a = ours[k].cpu().numpy()[em].view(np.uint32)  # bit patterns: NaN rows compare too
        b = ref[k].cpu().numpy()[em].view(np.uint32)
        same = (a == b).all(axis=1)
        print("  %s bit-exact rows %.6f" % (k, float(same.mean())))
        for i in np.flatnonzero(~same)[:5]:
            print("    gid %d ours %s ref %s" % (em[i], a[i].view(np.float32), b[i].view(np.float32)))
        assert same.all(), k


@pytest.mark.parametrize("case", list(CASES))
def test_sort_and_ranges_bit_exact_on_reference_keys(cuda_device, case):
    scene, spec, ref, _ = _run_both(case, True, cuda_device)
    M = int(ref["cnt"].item())
    W, H = spec.width, spec.height
    tiles = ((W + 15) // 16) * ((H + 15) // 16)
    ks, vs = torch.zeros_like(ref["keys"]), torch.zeros_like(ref["vals"])
    ws = torch.zeros(ops.get_sort_buffer_size(CAP), dtype=torch.int8, device=cuda_device)
    ops.sort_gaussian(M, W, H, 16, 16, ws, ref["keys"], ref["vals"], ks, vs)
    ek, ev = O.sort_pairs(_np(ref["keys"], M, np.uint64), _np(ref["vals"], M, np.uint32), O.end_bit_for(W, H))
    np.testing.assert_array_equal(_np(ks, M, np.uint64), ek)
    np.testing.assert_array_equal(_np(vs, M, np.uint32), ev)
    ours_r = torch.zeros((tiles, 2), dtype=torch.int32, device=cuda_device)
    ref_r = torch.zeros((tiles, 2), dtype=torch.int32, device=cuda_device)
    ops.precompute_tile_ranges(M, W, H, 16, 16, ks, ours_r)
    RK.tile_ranges(M, ks, tiles, ref_r)
    np.testing.assert_array_equal(ours_r.cpu().numpy(), ref_r.cpu().numpy())


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("which", ["lite", "fused", "default"])
def test_blend_vs_reference_same_inputs(cuda_device, case, which):
    scene, spec, ref, _ = _run_both(case, which != "default", cuda_device)
    M = int(ref["cnt"].item())
    W, H = spec.width, spec.height
    tiles = ((W + 15) // 16) * ((H + 15) // 16)
    ks, vs = torch.zeros_like(ref["keys"]), torch.zeros_like(ref["vals"])
    ws = torch.zeros(ops.get_sort_buffer_size(CAP), dtype=torch.int8, device=cuda_device)
    ops.sort_gaussian(M, W, H, 16, 16, ws, ref["keys"], ref["vals"], ks, vs)
    rr = torch.zeros((tiles, 2), dtype=torch.int32, device=cuda_device)
    ops.precompute_tile_ranges(M, W, H, 16, 16, ks, rr)
    bg = torch.tensor([0.2, 0.1, 0.6])
    out_ref = torch.zeros((H, W, 3), dtype=torch.uint8, device=cuda_device)
    out_gsr = torch.zeros_like(out_ref)
    RK.render(which, M, W, H, ref["xy"], ref["rgbd"], ref["con"], ks, vs, rr, bg.tolist(), out_ref)
    if which == "lite":
        ops.render_16x16_preranges_smem_persistent_lite(M, W, H, ref["xy"], ref["rgbd"], ref["con"], vs, rr, bg,
                                                        out_gsr)
    elif which == "fused":
        ops.render_16x16_preranges_smem_persistent_lite_fused(M, W, H, ref["xy"], ref["rgbd"], ref["con"], ks, vs,
                                                              bg, out_gsr)
    else:
        ops.render_16x16(M, W, H, ref["xy"], ref["rgbd"], ref["con"], ks, vs, bg, out_gsr)
    s = image_stats(out_gsr.cpu().numpy(), out_ref.cpu().numpy())
    print("\n%s %s: %s" % (case, which, s))
    assert s["max_abs"] <= 2 and s["psnr"] >= 50.0, s


@pytest.mark.parametrize("case", list(CASES))
def test_whole_frame_vs_reference(cuda_device, case):
    """The reference's pipeline end to end (its preprocess, its CUB sort call
    over bits [0, 32 + msb(tiles)), its ranges and its fused render) against
    this library's fused E2E forward."""
    from polysplat_gb300 import Rasterizer

    scene, spec, ref, _ = _run_both(case, True, cuda_device)
    M = int(ref["cnt"].item())
    W, H = spec.width, spec.height
    tiles = ((W + 15) // 16) * ((H + 15) // 16)
    ks, vs = torch.zeros_like(ref["keys"]), torch.zeros_like(ref["vals"])
    temp = torch.zeros(RK.sort_temp_bytes(M), dtype=torch.int8, device=cuda_device)
    msb = 16
    for step in (8, 4, 2, 1):  # getHigherMsb (sort.cu:14-29)
        msb = msb + step if tiles >> msb else msb - step
    if tiles >> msb:
        msb += 1
    RK.sort(M, 32 + msb, temp, ref["keys"], ref["vals"], ks, vs)
    rr = torch.zeros((tiles, 2), dtype=torch.int32, device=cuda_device)
    RK.tile_ranges(M, ks, tiles, rr)
    out_ref = torch.zeros((H, W, 3), dtype=torch.uint8, device=cuda_device)
    RK.render("fused", M, W, H, ref["xy"], ref["rgbd"], ref["con"], ks, vs, rr, [0.0, 0.0, 0.0], out_ref)
    rast = Rasterizer(scene, CAP, 1 << 16)
    img = rast.forward(scene, Camera.from_spec(spec), torch.zeros(3), render_variant="preranges_smem_persistent_lite_e2e")
    s = image_stats(img.cpu().numpy(), out_ref.cpu().numpy())
    print("\n%s whole frame vs reference: %s" % (case, s))
    assert s["max_abs"] <= 2 and s["psnr"] >= 50.0, s


@pytest.mark.slow
def test_city_20m_8k_frame_vs_reference(cuda_device):
    """city_20m_8k (20 M Gaussians, 7680x4320) end to end: the reference's own
    forward (its preprocess, CUB sort and fused render, RK.Pipeline) against
    this library's E2E forward.

    Both pipelines append keys with atomics, so Gaussians with equal depth
    bits in one tile reach the sort in an order neither fixes, and blend in
    that order (the reference differs from itself the same way between
    runs).  Bars: the sorted keys bit-identical; within every run of equal
    keys the same Gaussians (values equal as multisets); the images equal
    up to those runs' blend order, PSNR >= 60 dB with at most 1e-5 of the
    pixels different (the worst pixel is reported)."""
    from polysplat_gb300 import Rasterizer

    raw, cams = scenes.workload("city_20m_8k")
    scene = Scene.from_raw(raw, cuda_device)
    spec = cams[0]
    rast = Rasterizer(scene, 1 << 26, 1 << 18)
    img, st = rast.forward(scene, Camera.from_spec(spec), torch.zeros(3),
                           render_variant="preranges_smem_persistent_lite_e2e", return_stats=True)
    M = st["num_rendered"]
    img = img.cpu().numpy()
    ours = np.stack([rast.gaussian_keys_sorted[:M].cpu().numpy().view(np.uint64),
                     rast.gaussian_values_sorted[:M].cpu().numpy().view(np.uint32).astype(np.uint64)], axis=1)
    del rast
    torch.cuda.empty_cache()
    pipe = RK.Pipeline(scene, spec, 2 * M)
    n = pipe.forward()
    torch.cuda.synchronize()
    assert n == M, (n, M)
    ref = np.stack([pipe.ks[:M].cpu().numpy().view(np.uint64),
                    pipe.vs[:M].cpu().numpy().view(np.uint32).astype(np.uint64)], axis=1)
    assert np.array_equal(ours[:, 0], ref[:, 0]), int((ours[:, 0] != ref[:, 0]).sum())
    tied = int((ours[:, 1] != ref[:, 1]).sum())
    ours = ours[np.lexsort(ours.T[::-1])]
    ref = ref[np.lexsort(ref.T[::-1])]
    assert np.array_equal(ours, ref)
    s = image_stats(img, pipe.out.cpu().numpy())
    print("\ncity_20m_8k: %d keys bit-identical, %d positions hold another Gaussian of the same key run; image %s"
          % (M, tied, s))
    assert s["psnr"] >= 60.0 and s["frac_diff"] <= 1e-5, s
