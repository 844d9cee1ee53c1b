"""The large-Gaussian sweeps emit the tiles of a row's sure run (boxes deep
inside the ellipse) without running the exact tile test on them.  With
GSR_MASSIVE_SURE=0 every candidate tile gets the test.  Both must emit the
same (tile, Gaussian, depth) pairs, bit for bit, through every form that
sweeps queued Gaussians: the single-pass forward with per-tile and with quad
keys (warp and CTA sweeps), and the depth-first forward (counting pass,
emission and the wide-rectangle path).

The switch is read once per process, so the exhaustive side runs in a child
process and saves its key lists."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DUMP = r"""
import ctypes, sys
import numpy as np, torch
sys.path.insert(0, %(root)r)
sys.path.insert(0, %(tests)r)
from polysplat_gb300 import Camera, Scene, ops, scenes
from polysplat_gb300 import _lib as R
from polysplat_gb300._lib import check, lib

dev = torch.device("cuda:0")
CASES = [
    ("blobs_1080p", scenes.scene_blobs(4_000, seed=9), scenes.camera_front(1920, 1080, 1400.0)),
    ("blobs_odd", scenes.scene_blobs(3_000, seed=10), scenes.orbit_camera(7.0, 0.5, 0.2, 1000, 584, 700.0)),
    ("clustered_near", scenes.subsample(scenes.scene_clustered(600_000, seed=1), 150_000, seed=3),
     scenes.orbit_camera(3.5, 2.2, -0.3, 1920, 1080, 1400.0)),
    ("needles", scenes.scene_needles(60_000, seed=5), scenes.camera_front(1280, 720, 900.0)),
]
CAP = 1 << 24
out = {}
for name, raw, spec in CASES:
    scene, c = Scene.from_raw(raw, dev), Camera.from_spec(spec)
    P, W, H = scene.num_vertex, c.width, c.height
    T = ((W + 15) // 16) * ((H + 15) // 16)
    bg = torch.zeros(3)

    def bufs(key_dtype):
        z = lambda *s, dt=torch.float32: torch.zeros(s, dtype=dt, device=dev)
        return dict(curr=z(1, dt=torch.int32), ku=z(CAP, dt=key_dtype), vu=z(CAP, dt=torch.int32),
                    ks=z(CAP, dt=key_dtype), vs=z(CAP, dt=torch.int32), xy=z(P, 2), rgbd=z(P, 4), con=z(P, 4),
                    ranges=z(max(T, 1 << 17), 2, dt=torch.int32), img=z(H, W, 3, dt=torch.uint8),
                    ws=z(ops.get_sort_buffer_size(CAP), dt=torch.int8))

    for quad in (0, 0x100):
        f = bufs(torch.int64)
        f3 = ctypes.c_float * 3
        st = lib().gsr_forward(R.RENDER_PERSISTENT_RANGES | quad, P, scene.position.data_ptr(),
                               scene.shs_half.data_ptr(), 1, scene.opacity.data_ptr(), scene.cov3d.data_ptr(), W, H,
                               16, 16, f3(*c.position.tolist()), (ctypes.c_float * 9)(*c.rotation.reshape(-1).tolist()),
                               c.focal_x, c.focal_y, c.zFar, c.zNear, f["curr"].data_ptr(), f["ws"].data_ptr(),
                               f["ws"].numel(), f["ku"].data_ptr(), f["vu"].data_ptr(), f["ks"].data_ptr(),
                               f["vs"].data_ptr(), CAP, f["xy"].data_ptr(), f["rgbd"].data_ptr(), f["con"].data_ptr(),
                               f["ranges"].data_ptr(), f3(0.0, 0.0, 0.0), f["img"].data_ptr(),
                               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(st, "forward")
        n = ctypes.c_int32(0)
        check(lib().gsr_read_status(ctypes.c_void_p(f["ws"].data_ptr()), ctypes.c_void_p(f["curr"].data_ptr()), CAP,
                                    ctypes.byref(n), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
              "read_status")
        k = f["ku"][:n.value].cpu().numpy().view(np.uint64)
        v = f["vu"][:n.value].cpu().numpy().view(np.uint32)
        rows = np.stack([k, v.astype(np.uint64)], axis=1)
        out["%%s_single_%%d" %% (name, quad)] = rows[np.lexsort(rows.T[::-1])]
        out["%%s_image_%%d" %% (name, quad)] = f["img"].cpu().numpy()
    f = bufs(torch.int32)
    scratch = torch.zeros(ops.depth_first_scratch_size(P), dtype=torch.int8, device=dev)
    m = ops.forward_depth_first(R.RENDER_PERSISTENT_RANGES, True, scene.position, scene.shs_half, scene.opacity,
                                scene.cov3d, W, H, 16, 16, c.position, c.rotation, c.focal_x, c.focal_y, c.zFar,
                                c.zNear, f["curr"], f["ws"], scratch, f["ku"], f["vu"], f["ks"], f["vs"], f["xy"],
                                f["rgbd"], f["con"], f["ranges"][:T], bg, f["img"])
    out["%%s_df_tiles" %% name] = f["ks"][:m].cpu().numpy()
    out["%%s_df_vals" %% name] = f["vs"][:m].cpu().numpy()
torch.cuda.synchronize()
np.savez(sys.argv[1], **out)
"""


def _dump(path, sure):
    env = dict(os.environ)
    env["GSR_MASSIVE_SURE"] = "1" if sure else "0"
    code = DUMP % {"root": ROOT, "tests": os.path.join(ROOT, "tests")}
    r = subprocess.run([sys.executable, "-c", code, path], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    return np.load(path)


def test_sure_runs_emit_exactly_the_tested_tiles(tmp_path):
    fast = _dump(str(tmp_path / "sure.npz"), True)
    full = _dump(str(tmp_path / "tested.npz"), False)
    assert sorted(fast.files) == sorted(full.files)
    for k in sorted(fast.files):
        a, b = fast[k], full[k]
        assert a.shape == b.shape, (k, a.shape, b.shape)
        assert np.array_equal(a, b), (k, int((a != b).sum()))
    # the cases do queue large Gaussians: millions of pairs between them
    assert sum(fast[k].shape[0] for k in fast.files if "_single_0" in k) > 1_000_000
