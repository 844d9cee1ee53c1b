"""Generate the golden fixture of the reference's host-side code -- run where
the reference sources are (this container).

Every output comes from the reference's OWN code, compiled from its sources
by ``oracle/ref_host.py``:
* getViewMatrix / getProjectionMatrix (csrc/cuda_rasterizer/preprocess.cu:
  643-671) for 256 seeded cameras (random sizes, focal lengths, positions,
  orthonormal rotations; both clip planes of example.py:33-44 and others);
* loadPly_torch / computeCov3D (csrc/pybind.cpp:22-120) on a PLY written by
  ``scenes.write_ply`` from 1024 seeded Gaussians plus edge rows (extreme
  log-scales, opacity logits of +-30, quaternions of every sign and of tiny
  and huge norm).

The inputs are stored with the outputs.

    python tests/golden/make_host_golden.py [out_dir]      (default: tests/golden)
"""
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_host  # noqa: E402
from polysplat_gb300 import scenes  # noqa: E402


def cameras(n=256, seed=21):
    rng = np.random.default_rng(seed)
    W = rng.integers(16, 8000, n)
    H = rng.integers(16, 4500, n)
    fx = rng.uniform(50.0, 6000.0, n).astype(np.float32)
    fy = np.where(rng.random(n) < 0.5, fx, rng.uniform(50.0, 6000.0, n)).astype(np.float32)
    pos = rng.normal(0.0, 20.0, (n, 3)).astype(np.float32)
    rot = np.empty((n, 3, 3), np.float32)
    for i in range(n):
        q, r = np.linalg.qr(rng.normal(size=(3, 3)))
        rot[i] = (q * np.sign(np.diag(r))).astype(np.float32)
    zfar = np.where(rng.random(n) < 0.5, 100.0, rng.uniform(10.0, 1000.0, n)).astype(np.float32)
    znear = np.where(rng.random(n) < 0.5, 0.01, rng.uniform(0.001, 1.0, n)).astype(np.float32)
    return W.astype(np.int32), H.astype(np.int32), fx, fy, pos, rot, zfar, znear


def ply_scene():
    raw = scenes.scene_plain_small(1024, seed=22)
    means, ls, q, lg, shs = raw.means, raw.log_scales, raw.quats, raw.opacity_logits, raw.shs
    e_ls = np.array([[-12.0, -12.0, -12.0], [4.0, 4.0, 4.0], [-9.0, 2.0, 0.5], [3.0, -8.0, -1.0],
                     [0.0, 0.0, 0.0], [-3.5, -3.5, -3.5], [1.0, -1.0, 2.5], [-6.0, -6.0, 3.0]], np.float32)
    e_q = np.array([[1.0, 0.0, 0.0, 0.0], [-1.0, 0.0, 0.0, 0.0], [0.0, 0.0, 0.0, 1e-6], [5e3, -2e3, 7e3, 1e3],
                    [-0.3, 0.5, -0.7, 0.1], [1e-5, 2e-5, -3e-5, 4e-5], [0.5, 0.5, 0.5, 0.5], [0.0, -1.0, 0.0, 0.0]],
                   np.float32)
    e_lg = np.array([30.0, -30.0, 0.0, 8.0, -8.0, 1e-3, -17.5, 17.5], np.float32)
    k = len(e_lg)
    means = np.concatenate([means, np.random.default_rng(23).normal(0, 2, (k, 3)).astype(np.float32)])
    shs = np.concatenate([shs, np.random.default_rng(24).normal(0, 0.3, (k, 16, 3)).astype(np.float32)])
    return scenes.RawScene(means, np.concatenate([ls, e_ls]), np.concatenate([q, e_q]),
                           np.concatenate([lg, e_lg]), shs)


def main(out_dir):
    W, H, fx, fy, pos, rot, zfar, znear = cameras()
    views, projs = [], []
    for i in range(len(W)):
        v, p = ref_host.camera_matrices(W[i], H[i], pos[i], rot[i], fx[i], fy[i], zfar[i], znear[i])
        views.append(v)
        projs.append(p)
    raw = ply_scene()
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "scene.ply")
        scenes.write_ply(path, raw)
        r_pos, r_shs, r_op, r_cov = ref_host.load_ply(path, raw.num)
    np.savez_compressed(os.path.join(out_dir, "host_reference.npz"),
                        cam_W=W, cam_H=H, cam_fx=fx, cam_fy=fy, cam_pos=pos, cam_rot=rot, cam_zfar=zfar,
                        cam_znear=znear, ref_view=np.stack(views), ref_proj=np.stack(projs),
                        ply_means=raw.means, ply_log_scales=raw.log_scales, ply_quats=raw.quats,
                        ply_logits=raw.opacity_logits, ply_shs=raw.shs, ref_pos=r_pos, ref_shs=r_shs,
                        ref_opacity=r_op, ref_cov3d=r_cov)
    print("wrote", os.path.join(out_dir, "host_reference.npz"))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
