"""CPU checks of the FP64 oracle against independent numpy restatements and
known answers (no GPU needed)."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from polysplat_gb300 import scenes


def test_higher_msb_is_bit_length():
    # sort.cu:14-29 equals the number of bits needed to hold n for every n >= 1
    # (a frame always has at least one tile); for n = 0 it returns 1.
    for n in list(range(1, 70000)) + [129600, 2**20, 2**20 - 1, 2**31 - 1]:
        assert O.higher_msb(n) == int(n).bit_length(), n
    assert O.higher_msb(0) == 1


@pytest.mark.parametrize("tiles,expect", [(1900, 43), (3600, 44), (8160, 45), (14400, 46), (32400, 47),
                                          (129600, 49)])
def test_sort_width_per_resolution(tiles, expect):
    assert 32 + O.higher_msb(tiles) == expect


def _random_keys(rng, n, tiles, dup_frac=0.2):
    t = rng.integers(0, tiles, n).astype(np.uint64)
    d = rng.uniform(0.2, 60.0, n).astype(np.float32).view(np.uint32).astype(np.uint64)
    if n and dup_frac:
        k = int(n * dup_frac)
        d[:k] = d[0]  # many equal depths -> equal keys within a tile: stability matters
    return (t << np.uint64(32)) | d


@pytest.mark.parametrize("n", [0, 1, 7, 256, 4097, 50000])
@pytest.mark.parametrize("end_bit", [43, 45, 49, 64])
def test_sort_matches_numpy_stable(n, end_bit):
    rng = np.random.default_rng(n + end_bit)
    tiles = (1 << (end_bit - 32)) - 1 if end_bit < 64 else 1 << 20
    keys = _random_keys(rng, n, tiles)
    vals = rng.permutation(n).astype(np.uint32)
    ks, vs = O.sort_pairs(keys, vals, end_bit)
    masked = keys & np.uint64((1 << end_bit) - 1) if end_bit < 64 else keys
    order = np.argsort(masked, kind="stable")
    np.testing.assert_array_equal(ks, keys[order])
    np.testing.assert_array_equal(vs, vals[order])


def test_sort_ignores_bits_above_end_bit():
    keys = np.array([(5 << 40) | 3, 2, (1 << 50) | 1], dtype=np.uint64)
    vals = np.array([0, 1, 2], dtype=np.uint32)
    ks, vs = O.sort_pairs(keys, vals, 40)
    # bits >= 40 carried but ignored: order by low 40 bits = 1, 2, 3
    np.testing.assert_array_equal(vs, [2, 1, 0])
    np.testing.assert_array_equal(ks, keys[[2, 1, 0]])


@pytest.mark.parametrize("n,tiles", [(0, 10), (1, 1), (100, 7), (5000, 300), (20000, 8160)])
def test_tile_ranges_bsearch_and_scan(n, tiles):
    rng = np.random.default_rng(n * 31 + tiles)
    keys = np.sort(_random_keys(rng, n, max(1, tiles // 2) if tiles > 2 else tiles))
    r = O.tile_ranges(keys, tiles)
    hi = (keys >> np.uint64(32)).astype(np.int64)
    t = np.arange(tiles)
    np.testing.assert_array_equal(r[:, 0], np.searchsorted(hi, t, "left"))
    np.testing.assert_array_equal(r[:, 1], np.searchsorted(hi, t, "right"))
    s = O.tile_ranges(keys, tiles, scan=True)
    nonempty = r[:, 1] > r[:, 0]
    np.testing.assert_array_equal(s[nonempty], r[nonempty])
    assert not s[~nonempty].any()


def test_gather_known_answer():
    xy = np.arange(10, dtype=np.float32).reshape(5, 2)
    rgbd = np.arange(20, dtype=np.float32).reshape(5, 4)
    con = -np.arange(20, dtype=np.float32).reshape(5, 4)
    v = np.array([4, 0, 0, 2], dtype=np.uint32)
    a, b, c = O.gather(v, xy, rgbd, con)
    np.testing.assert_array_equal(a, xy[v])
    np.testing.assert_array_equal(b, rgbd[v])
    np.testing.assert_array_equal(c, con[v])


def _np_cov3d(log_scales, quats):
    s = np.exp(log_scales.astype(np.float64))
    q = quats.astype(np.float64)
    q = q / np.linalg.norm(q, axis=1, keepdims=True)
    r, x, y, z = q.T
    R = np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y)], -1),
                  np.stack([2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x)], -1),
                  np.stack([2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)], -1)], 1)
    M = R * s[:, None, :]
    S = M @ M.transpose(0, 2, 1)
    return np.stack([S[:, 0, 0], S[:, 0, 1], S[:, 0, 2], S[:, 1, 1], S[:, 1, 2], S[:, 2, 2]], 1)


def test_scene_transform_matches_numpy():
    sc = scenes.scene_plain_small(2000, seed=11)
    op, cov = O.scene_transform(sc.log_scales, sc.quats, sc.opacity_logits)
    np.testing.assert_allclose(op, 1 / (1 + np.exp(-sc.opacity_logits.astype(np.float64))), rtol=1e-6)
    np.testing.assert_allclose(cov, _np_cov3d(sc.log_scales, sc.quats), rtol=1e-5, atol=1e-12)


def _single_gaussian(x=0.0, y=0.0, z=0.0, scale=-1.0, logit=3.0, dc=(1.0, 0.5, 0.2)):
    means = np.array([[x, y, z]], np.float32)
    ls = np.full((1, 3), scale, np.float32)
    q = np.array([[1, 0, 0, 0]], np.float32)
    shs = np.zeros((1, 16, 3), np.float32)
    shs[0, 0] = dc
    return scenes.RawScene(means, ls, q, np.array([logit], np.float32), shs)


def test_preprocess_single_gaussian_known_answer():
    sc = _single_gaussian()
    op, cov = O.scene_transform(sc.log_scales, sc.quats, sc.opacity_logits)
    cam = scenes.camera_front(64, 48, 60.0)
    cp, cr = O.camera_args(cam)
    pre = O.preprocess(sc.means, sc.shs, op, cov, 64, 48, cp, cr, 60.0, 60.0)
    # centre projects to pixel ((W-1)/2, (H-1)/2) = (31.5, 23.5): tiles (1,1),(2,1)... key depth = 8
    np.testing.assert_allclose(pre["xy"][0], [31.5, 23.5], atol=1e-4)
    assert pre["rgbd"][0, 3] == np.float32(8.0)
    tiles = sorted(int(k >> np.uint64(32)) for k in pre["keys"])
    assert 1 * 4 + 1 in tiles  # tile (x=1, y=1) holds the centre (grid is 4x3)
    # colour = C0 * dc + 0.5 (direction along +z; higher orders are zero)
    np.testing.assert_allclose(pre["rgbd"][0, :3], 0.28209479177387814 * np.array([1.0, 0.5, 0.2]) + 0.5,
                               rtol=1e-6)
    # conic of the isotropic Gaussian: sigma_px^2 = (f*s/z)^2 + 0.3
    s2 = (60.0 * math.exp(-1.0) / 8.0) ** 2 + 0.3
    np.testing.assert_allclose(pre["con"][0, 0], -0.5 * math.log2(math.e) / s2, rtol=1e-5)


def test_culls_behind_near_plane():
    sc = _single_gaussian(z=-7.9)  # view depth 0.1 <= 0.2
    op, cov = O.scene_transform(sc.log_scales, sc.quats, sc.opacity_logits)
    cam = scenes.camera_front(64, 48, 60.0)
    cp, cr = O.camera_args(cam)
    pre = O.preprocess(sc.means, sc.shs, op, cov, 64, 48, cp, cr, 60.0, 60.0)
    assert pre["num"] == 0


def test_render_single_gaussian_analytic():
    # one Gaussian in one 16x16 tile: pixel = encode(rgb * alpha), alpha = 2^(con.w + quadratic)
    xy = np.array([[7.3, 8.6]], np.float32)
    con = np.array([[-0.05, 0.01, -0.04, math.log2(0.8)]], np.float32)
    rgbd = np.array([[0.9, 0.4, 0.1, 5.0]], np.float32)
    ranges = np.array([[0, 1]], np.int32)
    img = O.render(np.array([0], np.uint32), ranges, xy, rgbd, con, 16, 16, cadence=8)
    px, py = np.meshgrid(np.arange(16), np.arange(16))
    dx, dy = 7.3 - px, 8.6 - py
    a = 2.0 ** (con[0, 3] + con[0, 0] * dx * dx + con[0, 2] * dy * dy + con[0, 1] * dx * dy)
    expect = np.clip(a[..., None] * rgbd[0, :3] * 255.0, 0, 255).astype(np.uint8)
    np.testing.assert_array_equal(img, expect)


def test_render_saturation_exit_and_background():
    # 20 opaque copies: tile saturates; background only where T >= 1e-4
    n = 20
    xy = np.tile(np.array([[8.0, 8.0]], np.float32), (n, 1))
    con = np.tile(np.array([[-1e-6, 0.0, -1e-6, math.log2(0.999)]], np.float32), (n, 1))
    rgbd = np.tile(np.array([[0.5, 0.5, 0.5, 1.0]], np.float32), (n, 1))
    v = np.arange(n, dtype=np.uint32)
    img, cnt = O.render(v, np.array([[0, n]], np.int32), xy, rgbd, con, 16, 16, bg=(1.0, 1.0, 1.0),
                        cadence=2, want_counts=True)
    assert cnt[0] == 2  # T = 1e-6 after two Gaussians: all pixels saturate at the first check
    assert (img == np.uint8(0.5 * 0.999 * 255 + 0.5 * 0.999 * 0.001 * 255)).all()


def test_render_empty_tile_gets_background():
    img = O.render(np.zeros(0, np.uint32), np.zeros((4, 2), np.int32), np.zeros((1, 2), np.float32),
                   np.zeros((1, 4), np.float32), np.zeros((1, 4), np.float32), 20, 20, bg=(0.2, 0.6, 1.0))
    assert (img == np.array([51, 153, 255], np.uint8)).all()


def test_oracle_forward_deterministic_across_threads():
    sc = scenes.scene_plain_small(3000, seed=5)
    op, cov = O.scene_transform(sc.log_scales, sc.quats, sc.opacity_logits)
    cam = scenes.camera_front(160, 120, 120.0)
    a, pa = O.forward(sc.means, sc.shs, op, cov, cam, nthreads=1)
    b, pb = O.forward(sc.means, sc.shs, op, cov, cam, nthreads=5)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(pa["keys_sorted"], pb["keys_sorted"])


def test_masked_fp64_loss_gives_the_whole_image_differences():
    """The tile-masked FP64 loss (used for finite differences on large scenes):
    with every tile set it equals the whole-image loss bit for bit, and the
    central difference of one Gaussian's parameter over the tiles of its
    rectangle (grown by one tile) equals the whole image's."""
    raw = scenes.scene_plain_small(600, seed=9, mean_sigma=1.2)
    cam = scenes.orbit_camera(5.0, 0.4, 0.1, 160, 128, scenes.focal_for(160))
    target = O.image_fp64(raw.means + 0.03, raw.log_scales, raw.quats, raw.opacity_logits, raw.shs, cam)[1]
    full, img = O.image_fp64(raw.means, raw.log_scales, raw.quats, raw.opacity_logits, raw.shs, cam, target=target)
    gx, gy = (cam.width + 15) // 16, (cam.height + 15) // 16
    allm, imgm, rects = O.image_fp64_masked(raw.means, raw.log_scales, raw.quats, raw.opacity_logits, raw.shs,
                                            cam, np.ones(gx * gy, np.uint8), target=target)
    assert allm == full and np.array_equal(img, imgm)
    g = int(np.argmax((rects[:, 2] - rects[:, 0]) * (rects[:, 3] - rects[:, 1])))
    x0, y0, x1, y1 = rects[g]
    mask = np.zeros((gy, gx), np.uint8)
    mask[max(0, y0 - 1):min(gy, y1 + 1), max(0, x0 - 1):min(gx, x1 + 1)] = 1
    h = 1e-4
    means = raw.means.astype(np.float64)
    d_full, d_mask = [], []
    for sgn in (1, -1):
        m = means.copy()
        m[g, 0] += sgn * h
        d_full.append(O.image_fp64(m, raw.log_scales, raw.quats, raw.opacity_logits, raw.shs, cam, target=target)[0])
        d_mask.append(O.image_fp64_masked(m, raw.log_scales, raw.quats, raw.opacity_logits, raw.shs, cam,
                                          mask.reshape(-1), target=target)[0])
    fd_full = (d_full[0] - d_full[1]) / (2 * h)
    fd_mask = (d_mask[0] - d_mask[1]) / (2 * h)
    assert abs(fd_full - fd_mask) <= 1e-9 * max(1.0, abs(fd_full)), (fd_full, fd_mask)
