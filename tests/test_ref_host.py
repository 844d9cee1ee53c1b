"""The host-side parts of the path against the reference's own host code.

``tests/golden/host_reference.npz`` holds outputs of the reference's
getViewMatrix / getProjectionMatrix (csrc/cuda_rasterizer/preprocess.cu:
643-671) for 256 seeded cameras, and of its loadPly_torch / computeCov3D
(csrc/pybind.cpp:22-120) on a PLY of 1032 Gaussians, built from its sources
by oracle/ref_host.py (generator: tests/golden/make_host_golden.py).

* gsr_camera_matrices: bit-exact, view and projection, every camera;
* the PLY parse (positions, SH reordered to the interleaved layout):
  bit-exact;
* the FP64 oracle's scene transform: opacity within 2 ulp of the reference's
  FP32, each cov3d row within 2e-6 of its largest entry.
The device scene transform is checked against the same fixture in
tests/test_gpu_scene_prepare.py.
"""
import ctypes
import os

import numpy as np
import pytest

from polysplat_gb300 import ops, scenes
from polysplat_gb300._lib import lib

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "host_reference.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


def test_camera_matrices_bit_exact(gold):
    L = lib()
    f16 = ctypes.c_float * 16
    for i in range(len(gold["cam_W"])):
        view, proj = f16(), f16()
        L.gsr_camera_matrices(int(gold["cam_W"][i]), int(gold["cam_H"][i]),
                              (ctypes.c_float * 3)(*gold["cam_pos"][i].tolist()),
                              (ctypes.c_float * 9)(*gold["cam_rot"][i].reshape(-1).tolist()),
                              float(gold["cam_fx"][i]), float(gold["cam_fy"][i]), float(gold["cam_zfar"][i]),
                              float(gold["cam_znear"][i]), view, proj)
        v = np.array(view, np.float32).view(np.uint32)
        p = np.array(proj, np.float32).view(np.uint32)
        assert np.array_equal(v, gold["ref_view"][i].view(np.uint32)), i
        assert np.array_equal(p, gold["ref_proj"][i].view(np.uint32)), i


def _ply(gold, tmp_path):
    raw = scenes.RawScene(gold["ply_means"], gold["ply_log_scales"], gold["ply_quats"], gold["ply_logits"],
                          gold["ply_shs"])
    path = os.path.join(str(tmp_path), "scene.ply")
    scenes.write_ply(path, raw)
    return path


def test_ply_parse_bit_exact(gold, tmp_path):
    num, pos, shs, logits, log_scales, quats = ops.read_ply_raw(_ply(gold, tmp_path))
    assert num == gold["ref_pos"].shape[0]
    assert np.array_equal(pos.view(np.uint32), gold["ref_pos"].view(np.uint32))
    assert np.array_equal(shs.reshape(num, 48).view(np.uint32), gold["ref_shs"].view(np.uint32))
    assert np.array_equal(logits, gold["ply_logits"]) and np.array_equal(quats, gold["ply_quats"])


def test_oracle_scene_transform_vs_reference(gold):
    from oracle import oracle as O

    op, cov = O.scene_transform(gold["ply_log_scales"], gold["ply_quats"], gold["ply_logits"])
    ulp = np.abs(op.view(np.int32).astype(np.int64) - gold["ref_opacity"].view(np.int32).astype(np.int64))
    assert ulp.max() <= 2, ulp.max()
    scale = np.abs(gold["ref_cov3d"]).max(axis=1, keepdims=True)
    err = np.abs(cov.astype(np.float64) - gold["ref_cov3d"]) / scale
    assert err.max() <= 2e-6, err.max()
