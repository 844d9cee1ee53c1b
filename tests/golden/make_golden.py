"""Generate the golden fixtures of the reference rasterizer -- run on a GB300.

Every output here comes from the reference's OWN code: its preprocess,
tile-range and render kernels compiled from its sources (oracle/ref_build.py)
and launched by oracle/refrun.cu, and its sort call (CUB
DeviceRadixSort::SortPairs over bits [0, 32+msb(tiles)), sort.cu:107-125).
The inputs are stored with the outputs so the fixtures do not depend on the
random-number stream of the numpy that regenerates them.

    python tests/golden/make_golden.py [out_dir]      (default: tests/golden)

Each case file ref_<case>.npz holds: pos, shs (fp32 [P,48]), opacity, cov3d,
camera (W, H, fx, fy, position, rotation), bg; for sh in {fp32, fp16}:
num_<sh>, keys_sorted_<sh>, vals_sorted_<sh>, keys_unsorted_<sh>,
vals_unsorted_<sh>, xy_<sh>, rgbd_<sh>, con_<sh>, emitted_<sh> (Gaussians
with keys); ranges_fp16 (computeTileRanges); img_lite, img_fused,
img_default (renders of the fp16 lists, cadence 8 / 16 / 2).
"""
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import refkernels as RK  # noqa: E402
from polysplat_gb300 import Scene, scenes  # noqa: E402


def cases():
    small = scenes.subsample(scenes.scene_plain_small(), 2000, seed=11)
    heavy = scenes.subsample(scenes.scene_clustered(400_000, seed=1), 2000, seed=12)
    orbit = scenes.subsample(scenes.scene_clustered(400_000, seed=5), 2000, seed=13)
    return {
        "plain_256x192": (small, scenes.camera_front(256, 192, 192.0)),
        "heavy_320x180": (heavy, scenes.camera_front(320, 180, 1400.0 / 6)),
        "orbit_320x240": (orbit, scenes.orbit_camera(8.0, 0.9, 0.25, 320, 240, 300.0)),
    }


def run_case(raw, cam, dev):
    scene = Scene.from_raw(raw, dev)
    P = raw.num
    W, H = cam.width, cam.height
    tiles = ((W + 15) // 16) * ((H + 15) // 16)
    end_bit = 32 + tiles.bit_length()
    cap = 1 << 20
    out = dict(pos=raw.means, shs=raw.shs.reshape(P, 48), opacity=scene.opacity.cpu().numpy(),
               cov3d=scene.cov3d.cpu().numpy(), W=W, H=H, fx=cam.fx, fy=cam.fy, position=cam.position,
               rotation=cam.rotation, bg=np.array([0.1, 0.2, 0.3], np.float32))
    for sh, half in (("fp32", False), ("fp16", True)):
        xy = torch.zeros((P, 2), device=dev)
        rgbd = torch.zeros((P, 4), device=dev)
        con = torch.zeros((P, 4), device=dev)
        cnt = torch.zeros(1, dtype=torch.int32, device=dev)
        ku = torch.zeros(cap, dtype=torch.int64, device=dev)
        vu = torch.zeros(cap, dtype=torch.int32, device=dev)
        RK.preprocess(scene, cam, half, xy, scene.cov3d, rgbd, con, cnt, ku, vu)
        torch.cuda.synchronize()
        n = int(cnt.item())
        assert n < cap // 4, n
        ks, vs = torch.zeros_like(ku), torch.zeros_like(vu)
        temp = torch.zeros(RK.sort_temp_bytes(n), dtype=torch.int8, device=dev)
        RK.sort(n, end_bit, temp, ku, vu, ks, vs)
        torch.cuda.synchronize()
        vals = vs[:n].cpu().numpy().view(np.uint32)
        emitted = np.zeros(P, bool)
        emitted[np.unique(vals)] = True
        out.update({"num_" + sh: n, "keys_sorted_" + sh: ks[:n].cpu().numpy().view(np.uint64),
                    "vals_sorted_" + sh: vals, "keys_unsorted_" + sh: ku[:n].cpu().numpy().view(np.uint64),
                    "vals_unsorted_" + sh: vu[:n].cpu().numpy().view(np.uint32),
                    "xy_" + sh: xy.cpu().numpy(), "rgbd_" + sh: rgbd.cpu().numpy(), "con_" + sh: con.cpu().numpy(),
                    "emitted_" + sh: emitted})
        if half:
            rr = torch.zeros((tiles, 2), dtype=torch.int32, device=dev)
            RK.tile_ranges(n, ks, tiles, rr)
            out["ranges_fp16"] = rr.cpu().numpy()
            for which in ("lite", "fused", "default"):
                img = torch.zeros((H, W, 3), dtype=torch.uint8, device=dev)
                RK.render(which, n, W, H, xy, rgbd, con, ks, vs, rr, out["bg"].tolist(), img)
                torch.cuda.synchronize()
                out["img_" + which] = img.cpu().numpy()
    return out


def main():
    out_dir = sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__))
    os.makedirs(out_dir, exist_ok=True)
    dev = torch.device("cuda", 0)
    for name, (raw, cam) in cases().items():
        d = run_case(raw, cam, dev)
        np.savez_compressed(os.path.join(out_dir, "ref_%s.npz" % name), **d)
        print(name, "M(fp16)=%d M(fp32)=%d" % (d["num_fp16"], d["num_fp32"]))


if __name__ == "__main__":
    main()
