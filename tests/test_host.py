"""CPU tests of the host side: the C-ABI library loads and exports every
declared symbol, the ops mirror exposes the reference's 43 positional-only
operators, the PLY reader, and the synthetic workloads (no GPU calls)."""
import ctypes
import inspect
import os
import re

import numpy as np
import pytest

from polysplat_gb300 import build, ops, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

REFERENCE_OPS = [
    "loadPly", "preprocess", "preprocess_half_sh", "preprocess_es_pass_a", "preprocess_es_pass_a_half_sh",
    "preprocess_es_pass_b", "es_depth_sort_and_scan", "es_tile_sort", "get_es_scan_buffer_size",
    "sort_gaussian", "get_sort_buffer_size", "gather_features", "render_16x16", "render_16x16_preranges",
    "render_16x16_preranges_smem", "render_16x16_preranges_smem_persistent",
    "render_16x16_preranges_smem_persistent_lite", "render_16x16_preranges_smem_persistent_lite_dt",
    "render_16x16_preranges_naive", "render_16x16_preranges_smem_v2", "render_16x16_topk_smem",
    "render_16x16_topk_smem_persistent", "render_16x16_topk_smem_persistent_v2", "precompute_tile_ranges",
    "precompute_tile_ranges_scan", "compute_tile_order", "get_tile_order_sort_temp_size",
    "render_16x16_reordered", "compute_tile_order_packed", "compute_tile_order_packed_morton",
    "render_16x16_reordered_v2", "render_16x16_reordered_persistent", "render_16x16_unroll2",
    "render_16x16_split", "render_24x16_split", "render_32x16", "render_32x16_split", "render_32x32",
    "sort_and_render", "forward_fused", "render_16x16_preranges_smem_persistent_lite_fused",
    "forward_fused_e2e", "forward_fused_e2e_preranges",
]


def _declared_symbols():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^\s*(?:gsr_status|size_t|int|void)\s+(gsr_\w+)\s*\(", src, re.M)
    return sorted(set(names))


def test_library_builds_and_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    names = _declared_symbols()
    assert len(names) >= 13
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_library_is_built_for_sm103a_only():
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_ops_has_the_43_reference_operators():
    assert len(REFERENCE_OPS) == 43
    for name in REFERENCE_OPS:
        fn = getattr(ops, name)
        assert callable(fn), name
    assert sorted(ops.__all__) == sorted(REFERENCE_OPS)


@pytest.mark.parametrize("name", [n for n in REFERENCE_OPS if not n.startswith("preprocess_es")
                                  and not n.startswith("es_")])
def test_ops_take_positional_only_arguments(name):
    sig = inspect.signature(getattr(ops, name))
    kinds = {p.kind for p in sig.parameters.values()}
    assert kinds <= {inspect.Parameter.POSITIONAL_ONLY}, (name, kinds)


def test_fused_signatures_match_reference_arity():
    # csrc/pybind.cpp:1085-1095, 932-943, 1016-1026, 876-886
    assert len(inspect.signature(ops.forward_fused_e2e).parameters) == 25
    assert len(inspect.signature(ops.forward_fused).parameters) == 26
    assert len(inspect.signature(ops.forward_fused_e2e_preranges).parameters) == 26
    assert len(inspect.signature(ops.sort_and_render).parameters) == 16
    assert len(inspect.signature(ops.preprocess).parameters) == 20
    assert len(inspect.signature(ops.sort_gaussian).parameters) == 10


def test_ply_roundtrip_parse(tmp_path):
    sc = scenes.scene_plain_small(257, seed=3)
    p = str(tmp_path / "a.ply")
    scenes.write_ply(p, sc)
    num, pos, shs, logits, ls, q = ops.read_ply_raw(p)
    assert num == 257
    np.testing.assert_array_equal(pos, sc.means)
    np.testing.assert_array_equal(shs, sc.shs)
    np.testing.assert_array_equal(logits, sc.opacity_logits)
    np.testing.assert_array_equal(ls, sc.log_scales)
    np.testing.assert_array_equal(q, sc.quats)


def test_ply_errors(tmp_path):
    p = tmp_path / "bad.ply"
    p.write_bytes(b"ply\nformat binary_little_endian 1.0\nelement vertex 0\n")
    with pytest.raises(RuntimeError):
        ops.read_ply_raw(str(p))
    p.write_bytes(b"ply\nelement vertex 5\nend_header\n" + b"\0" * 40)
    with pytest.raises(RuntimeError):
        ops.read_ply_raw(str(p))


def test_workloads_are_deterministic():
    a = scenes.scene_clustered(5000, seed=1)
    b = scenes.scene_clustered(5000, seed=1)
    np.testing.assert_array_equal(a.means, b.means)
    np.testing.assert_array_equal(a.shs, b.shs)
    assert a.means.dtype == np.float32 and a.shs.shape == (5000, 16, 3)
    q = a.quats
    np.testing.assert_allclose(np.linalg.norm(q, axis=1), 1.0, rtol=1e-5)


def test_look_at_identity_matches_front_camera():
    c = scenes.look_at([0, 0, -8], [0, 0, 0], 800, 600, 600.0, 600.0)
    np.testing.assert_allclose(c.rotation, np.eye(3), atol=1e-7)


def test_serve_mix_shape():
    sc, reqs = scenes.serve_mix(num_requests=64, scene_sizes=(1000, 2000))
    assert len(sc) == 2 and len(reqs) == 64
    t = [r.arrival_s for r in reqs]
    assert all(b > a for a, b in zip(t, t[1:]))
    assert {(r.camera.width, r.camera.height) for r in reqs} <= set(scenes.RESOLUTIONS)


def test_training_view_cameras_pack_as_the_c_abi_reads_them():
    """gsr_train_forward_views / gsr_train_backward_views read host arrays
    cam_pos [V,3], cam_rot [V,9] (row-major, as cameras.json) and cam_intr
    [V,4] = (focal_x, focal_y, z_far, z_near), view after view."""
    import math

    from polysplat_gb300.diff import _views_cam_args
    from polysplat_gb300.rasterizer import Camera

    cams = [Camera.from_spec(scenes.orbit_camera(10.0, 2 * math.pi * k / 3, 0.1 * k, 320, 180, 200.0 + k, id=k))
            for k in range(3)]
    pos, rot, intr = _views_cam_args(cams)
    assert (len(pos), len(rot), len(intr)) == (9, 27, 12)
    for v, c in enumerate(cams):
        assert np.allclose(np.array(pos[3 * v:3 * v + 3]), c.position.numpy().reshape(-1))
        assert np.allclose(np.array(rot[9 * v:9 * v + 9]), c.rotation.numpy().reshape(-1))
        assert np.allclose(np.array(intr[4 * v:4 * v + 4]), [c.focal_x, c.focal_y, c.zFar, c.zNear])
