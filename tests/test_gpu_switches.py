"""The library's two process-wide kernel switches give the same results as
the defaults on the same inputs, bit for bit:

* GSR_SORT_RANK=ballot / match: digit ranking by per-bit ballots, or by
  match.any, on every pass (the default picks per pass).  Stable sorts of
  the same pairs, so keys and values must be equal.
* GSR_RENDER_TMA=1: the render stages its Gaussian batches with 16-byte
  cp.async.bulk copies completed on an mbarrier instead of per-thread
  cp.async.  The blend is the same, so images must be equal.

A switch is read once per process, so each one runs in a child process on
inputs this process made and saved."""
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from polysplat_gb300 import Camera, Scene, ops, scenes

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RENDERS = ("render_16x16_preranges_smem_persistent_lite", "render_16x16_preranges_smem_persistent_lite_fused",
           "render_16x16", "render_16x16_split")

CHILD = r"""
import sys, numpy as np, torch
sys.path.insert(0, %(root)r)
from polysplat_gb300 import ops
dev = torch.device("cuda:0")
f = np.load(%(inp)r)
n, W, H = int(f["n"]), int(f["W"]), int(f["H"])
g = lambda k: torch.from_numpy(f[k]).to(dev)
ku, vu = g("ku"), g("vu")
ks, vs = torch.zeros_like(ku), torch.zeros_like(vu)
ws = torch.zeros(ops.get_sort_buffer_size(n), dtype=torch.int8, device=dev)
ops.sort_gaussian(n, W, H, 16, 16, ws, ku, vu, ks, vs)
out = {"ks": ks.cpu().numpy(), "vs": vs.cpu().numpy()}
xy, rgbd, con, rb = g("xy"), g("rgbd"), g("con"), g("rb")
ks0, vs0 = g("ks"), g("vs")
bg = torch.tensor([0.1, 0.2, 0.3])
for name in %(renders)r:
    img = torch.zeros((H, W, 3), dtype=torch.uint8, device=dev)
    fn = getattr(ops, name)
    if "preranges" in name and "fused" not in name:
        fn(n, W, H, xy, rgbd, con, vs0, rb, bg, img)
    else:
        fn(n, W, H, xy, rgbd, con, ks0, vs0, bg, img)
    out[name] = img.cpu().numpy()
torch.cuda.synchronize()
np.savez(%(outp)r, **out)
"""


@pytest.fixture(scope="module")
def frame(tmp_path_factory):
    dev = torch.device("cuda:0")
    raw = scenes.scene_clustered(200_000, seed=12)
    c = Camera.from_spec(scenes.orbit_camera(8.0, 0.4, 0.2, 1920, 1080, scenes.focal_for(1920)))
    scene = Scene.from_raw(raw, dev)
    W, H, P, cap = c.width, c.height, scene.num_vertex, 1 << 23
    ku = torch.zeros(cap, dtype=torch.int64, device=dev)
    vu = torch.zeros(cap, dtype=torch.int32, device=dev)
    xy, rgbd, con = (torch.zeros((P, k), device=dev) for k in (2, 4, 4))
    cnt = torch.zeros(1, dtype=torch.int32, device=dev)
    ops.preprocess_half_sh(scene.position, scene.shs_half, scene.opacity, scene.cov3d, W, H, 16, 16, c.position,
                           c.rotation, c.focal_x, c.focal_y, c.zFar, c.zNear, xy, rgbd, con, ku, vu, cnt)
    n = int(cnt.item())
    ku, vu = ku[:n].clone(), vu[:n].clone()
    ks, vs = torch.zeros_like(ku), torch.zeros_like(vu)
    ws = torch.zeros(ops.get_sort_buffer_size(n), dtype=torch.int8, device=dev)
    ops.sort_gaussian(n, W, H, 16, 16, ws, ku, vu, ks, vs)
    T = ((W + 15) // 16) * ((H + 15) // 16)
    rb = torch.zeros((T, 2), dtype=torch.int32, device=dev)
    ops.precompute_tile_ranges(n, W, H, 16, 16, ks, rb)
    bg = torch.tensor([0.1, 0.2, 0.3])
    images = {}
    for name in RENDERS:
        img = torch.zeros((H, W, 3), dtype=torch.uint8, device=dev)
        fn = getattr(ops, name)
        if "preranges" in name and "fused" not in name:
            fn(n, W, H, xy, rgbd, con, vs, rb, bg, img)
        else:
            fn(n, W, H, xy, rgbd, con, ks, vs, bg, img)
        images[name] = img.cpu().numpy()
    path = str(tmp_path_factory.mktemp("switches") / "inputs.npz")
    arrays = dict(n=n, W=W, H=H, ku=ku, vu=vu, ks=ks, vs=vs, xy=xy, rgbd=rgbd, con=con, rb=rb)
    np.savez(path, **{k: (v.cpu().numpy() if torch.is_tensor(v) else v) for k, v in arrays.items()})
    return dict(path=path, n=n, ks=ks.cpu().numpy(), vs=vs.cpu().numpy(), images=images)


def _child(frame, env_extra, tmp_path):
    outp = str(tmp_path / "out.npz")
    env = dict(os.environ)
    env.pop("GSR_SORT_RANK", None)
    env.pop("GSR_RENDER_TMA", None)
    env.update(env_extra)
    script = CHILD % dict(root=ROOT, inp=frame["path"], outp=outp, renders=RENDERS)
    r = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return np.load(outp)


@pytest.mark.parametrize("env", [{"GSR_SORT_RANK": "ballot"}, {"GSR_SORT_RANK": "match"}, {"GSR_RENDER_TMA": "1"}],
                         ids=["rank_ballot", "rank_match", "render_tma"])
def test_switch_gives_identical_results(frame, env, tmp_path):
    got = _child(frame, env, tmp_path)
    assert frame["n"] > 300_000  # about 130 sort tiles of 4096 keys
    assert np.array_equal(got["ks"], frame["ks"]) and np.array_equal(got["vs"], frame["vs"])
    for name in RENDERS:
        assert np.array_equal(got[name], frame["images"][name]), name
