"""CPU pinning of the FP64 oracle against golden outputs of the REFERENCE's own
code (its preprocess / tile-range / render kernels and its CUB sort call, run
on a GB300 by tests/golden/make_golden.py).  No GPU needed.

  * sort: the oracle's stable LSD radix sort of the reference's unsorted keys
    equals CUB's output bit for bit (keys and values, ties included);
  * tile ranges: bit-exact against computeTileRanges;
  * blend: the oracle's FP64 blend of the reference's lists and features is
    within max-abs 2/255 and PSNR >= 50 dB of each reference render kernel;
  * preprocess: on the well-conditioned scene the oracle's key set equals the
    reference's; on the heavy-tailed scenes the FP64-vs-FP32 error is stated.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

from helpers import compare_key_lists, image_stats

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FILES = sorted(glob.glob(os.path.join(HERE, "ref_*.npz")))


def _load(path):
    return dict(np.load(path))


def _tiles(d):
    return ((int(d["W"]) + 15) // 16) * ((int(d["H"]) + 15) // 16)


def test_goldens_present():
    assert len(FILES) >= 3


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
@pytest.mark.parametrize("sh", ["fp16", "fp32"])
def test_oracle_sort_equals_reference_cub(path, sh):
    d = _load(path)
    eb = O.end_bit_for(int(d["W"]), int(d["H"]))
    ks, vs = O.sort_pairs(d["keys_unsorted_" + sh], d["vals_unsorted_" + sh], eb)
    np.testing.assert_array_equal(ks, d["keys_sorted_" + sh])
    np.testing.assert_array_equal(vs, d["vals_sorted_" + sh])


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
def test_oracle_tile_ranges_equal_reference(path):
    d = _load(path)
    r = O.tile_ranges(d["keys_sorted_fp16"], _tiles(d))
    np.testing.assert_array_equal(r, d["ranges_fp16"])


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
@pytest.mark.parametrize("which,cadence", [("lite", 8), ("fused", 16), ("default", 2)])
def test_oracle_blend_matches_reference_render(path, which, cadence):
    d = _load(path)
    img = O.render(d["vals_sorted_fp16"], d["ranges_fp16"], d["xy_fp16"], d["rgbd_fp16"], d["con_fp16"],
                   int(d["W"]), int(d["H"]), d["bg"], cadence=cadence)
    s = image_stats(img, d["img_" + which])
    assert s["max_abs"] <= 2 and s["psnr"] >= 50.0, s


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
@pytest.mark.parametrize("sh", ["fp16", "fp32"])
def test_oracle_preprocess_vs_reference(path, sh):
    d = _load(path)
    shs = d["shs"]
    if sh == "fp16":
        shs = shs.astype(np.float16).astype(np.float32)
    pre = O.preprocess(d["pos"], shs, d["opacity"], d["cov3d"], int(d["W"]), int(d["H"]),
                       d["position"], d["rotation"].reshape(9), float(d["fx"]), float(d["fy"]))
    rk, rv = d["keys_sorted_" + sh], d["vals_sorted_" + sh]
    only_o, only_r, ulp = compare_key_lists(pre["keys"], pre["vals"], rk, rv)
    print("\n%s %s: M_ref=%d M_fp64=%d only_fp64=%d only_ref=%d depth_ulp=%d"
          % (os.path.basename(path), sh, rk.size, pre["num"], only_o, only_r, ulp))
    cov_ok = np.isfinite(d["cov3d"]).all(axis=1)
    if "plain" in path:
        # well-conditioned: exact key set, depths within 2 ulp, features close
        assert only_o == 0 and only_r == 0 and ulp <= 2
        em = d["emitted_" + sh] & pre["emitted"] & cov_ok
        assert np.abs(pre["xy"][em] - d["xy_" + sh][em]).max() <= 2e-3
        for k in ("rgbd", "con"):
            a, b = pre[k][em], d[k + "_" + sh][em]
            assert (np.abs(a - b) <= 1e-5 + 1e-4 * np.abs(b)).all(), k
    else:
        # stated error on heavy-tailed scales; bounded loosely
        assert only_o + only_r <= max(16, 0.2 * rk.size)


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
def test_oracle_forward_vs_reference_image(path):
    """Whole FP64 frame vs the reference's fused render: stated per case,
    and within the image bar on the well-conditioned scene."""
    d = _load(path)

    class Cam:
        pass

    cam = Cam()
    cam.width, cam.height = int(d["W"]), int(d["H"])
    cam.fx, cam.fy = float(d["fx"]), float(d["fy"])
    cam.position, cam.rotation = d["position"], d["rotation"]
    img, pre = O.forward(d["pos"], d["shs"], d["opacity"], d["cov3d"], cam, bg=d["bg"], cadence=16, half_sh=True)
    s = image_stats(img, d["img_fused"])
    print("\n%s FP64 forward vs reference: %s" % (os.path.basename(path), s))
    if "plain" in path:
        assert s["max_abs"] <= 2 and s["psnr"] >= 50.0, s
