"""Quad keys (GSR_QUAD_KEYS): one sort key per 2x2 group of 16x16 tiles, with
the hit tiles as a mask in the value, against the per-tile pipeline.

Bars (integer and index work, so bit-exact):
* the quad keys, expanded to (tile, Gaussian, depth bits) triples through
  their masks, are exactly the per-tile emission's triples, through every
  emission scheme (single tile, per-warp pool, queued CTA and warp sweeps,
  and the in-place sweep when the large-Gaussian queue is full);
* the image is bit-identical to the per-tile forward's, for the exit
  cadences 16 (E2E), 8 (lite) and 2 (default), single view and batched;
* on the reference's own kernels (where built) the quad image equals the
  reference's E2E image.
"""
import ctypes

import numpy as np
import pytest
import torch

from polysplat_gb300 import Camera, Scene, scenes
from polysplat_gb300 import _lib as R
from polysplat_gb300._lib import check, lib
from polysplat_gb300.batch import Batcher, View

pytestmark = pytest.mark.gpu

QUAD = 0x100  # GSR_QUAD_KEYS


class _Frame:
    """Buffers of one single-view forward through the C ABI."""

    def __init__(self, scene, cap, dev):
        P = scene.num_vertex
        self.scene, self.cap, self.dev = scene, cap, dev
        self.ku = torch.zeros(cap, dtype=torch.int64, device=dev)
        self.vu = torch.zeros(cap, dtype=torch.int32, device=dev)
        self.ks = torch.zeros(cap, dtype=torch.int64, device=dev)
        self.vs = torch.zeros(cap, dtype=torch.int32, device=dev)
        self.xy = torch.zeros((P, 2), device=dev)
        self.rgbd = torch.zeros((P, 4), device=dev)
        self.con = torch.zeros((P, 4), device=dev)
        self.ctr = torch.zeros(1, dtype=torch.int32, device=dev)
        self.ws = torch.zeros(lib().gsr_workspace_size(cap), dtype=torch.int8, device=dev)
        self.ranges = torch.zeros((1 << 17, 2), dtype=torch.int32, device=dev)

    def forward(self, cam, variant, bg=(0.0, 0.0, 0.0)):
        s = self.scene
        out = torch.zeros((cam.height, cam.width, 3), dtype=torch.uint8, device=self.dev)
        f3 = (ctypes.c_float * 3)
        st = lib().gsr_forward(variant, s.num_vertex, s.position.data_ptr(), s.shs_half.data_ptr(), 1,
                               s.opacity.data_ptr(), s.cov3d.data_ptr(), cam.width, cam.height, 16, 16,
                               f3(*cam.position.tolist()), (ctypes.c_float * 9)(*cam.rotation.reshape(-1).tolist()),
                               cam.focal_x, cam.focal_y, cam.zFar, cam.zNear, self.ctr.data_ptr(),
                               self.ws.data_ptr(), self.ws.numel(), self.ku.data_ptr(), self.vu.data_ptr(),
                               self.ks.data_ptr(), self.vs.data_ptr(), self.cap, self.xy.data_ptr(),
                               self.rgbd.data_ptr(), self.con.data_ptr(), self.ranges.data_ptr(), f3(*bg),
                               out.data_ptr(), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(st, "forward")
        n = ctypes.c_int32(0)
        st = lib().gsr_read_status(ctypes.c_void_p(self.ws.data_ptr()), ctypes.c_void_p(self.ctr.data_ptr()),
                                   self.cap, ctypes.byref(n), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(st, "read_status", n.value)
        M = n.value
        keys = self.ku[:M].cpu().numpy().view(np.uint64).copy()
        vals = self.vu[:M].cpu().numpy().view(np.uint32).copy()
        sk = self.ks[:M].cpu().numpy().view(np.uint64).copy()
        return out, keys, vals, sk


class _DevWords:
    """int32 view of library-owned device words."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i4", "data": (int(ptr), False), "version": 3,
                                         "strides": None}


def _expand_quads(keys, vals, gx):
    """(tile, gaussian, depth) triples of quad keys, tile = y * gx + x."""
    qgx = (gx + 1) // 2
    q = (keys >> np.uint64(32)).astype(np.int64)
    d = (keys & np.uint64(0xFFFFFFFF)).astype(np.int64)
    m = (vals >> np.uint32(28)).astype(np.int64)
    g = (vals & np.uint32((1 << 28) - 1)).astype(np.int64)
    assert (m > 0).all(), "a quad key without a hit tile"
    out = []
    for s in range(4):
        sel = (m >> s) & 1 == 1
        x = 2 * (q[sel] % qgx) + (s & 1)
        y = 2 * (q[sel] // qgx) + (s >> 1)
        out.append(np.stack([y * gx + x, g[sel], d[sel]], axis=1))
    return np.concatenate(out)


def _per_tile(keys, vals):
    t = (keys >> np.uint64(32)).astype(np.int64)
    d = (keys & np.uint64(0xFFFFFFFF)).astype(np.int64)
    return np.stack([t, vals.astype(np.int64), d], axis=1)


def _sorted_rows(a):
    return a[np.lexsort(a.T[::-1])]


def _cases():
    clustered = scenes.subsample(scenes.scene_clustered(600_000, seed=1), 120_000, seed=3)
    return [
        ("plain", scenes.subsample(scenes.scene_plain_small(), 40_000, seed=1), scenes.camera_front(800, 600, 600.0)),
        # odd tile columns and rows: quads cut by the image edge
        ("clustered_odd", clustered, scenes.orbit_camera(9.0, 0.8, 0.2, 1000, 584, scenes.focal_for(1000))),
        ("clustered_1080p", clustered, scenes.camera_front(1920, 1080, 1400.0)),
        ("needles", scenes.scene_needles(60_000, seed=5), scenes.camera_front(1272, 712, 900.0)),
    ]


@pytest.mark.parametrize("name,raw,spec", _cases(), ids=[c[0] for c in _cases()])
def test_quad_keys_expand_to_per_tile_keys_and_same_image(cuda_device, name, raw, spec):
    scene = Scene.from_raw(raw, cuda_device)
    cam = Camera.from_spec(spec)
    fr = _Frame(scene, 8_000_000, cuda_device)
    gx = (cam.width + 15) // 16
    for variant in (R.RENDER_PERSISTENT_FUSED, R.RENDER_PERSISTENT_RANGES, R.RENDER_DEFAULT):
        img_t, kt, vt, _ = fr.forward(cam, variant)
        img_t = img_t.clone()
        img_q, kq, vq, sq = fr.forward(cam, variant | QUAD)
        assert torch.equal(img_q, img_t), (name, variant, int((img_q != img_t).sum()))
    # emission: exact triple sets (the last variant's keys)
    assert len(kq) < len(kt)
    assert np.array_equal(_sorted_rows(_expand_quads(kq, vq, gx)), _sorted_rows(_per_tile(kt, vt)))
    # the sorted quad keys are in (quad, depth) order
    assert np.all(sq[1:] >= sq[:-1])


def _depth_first(fr, cam, variant, scratch):
    """gsr_forward_depth_first on the frame's buffers (32-bit tile ids in the
    key buffers' front halves); returns (image, M, sorted tile ids, values)."""
    s = fr.scene
    out = torch.zeros((cam.height, cam.width, 3), dtype=torch.uint8, device=fr.dev)
    f3 = (ctypes.c_float * 3)
    tu, ts = fr.ku.view(torch.int32), fr.ks.view(torch.int32)
    st = lib().gsr_forward_depth_first(
        variant, s.num_vertex, s.position.data_ptr(), s.shs_half.data_ptr(), 1, s.opacity.data_ptr(),
        s.cov3d.data_ptr(), cam.width, cam.height, 16, 16, f3(*cam.position.tolist()),
        (ctypes.c_float * 9)(*cam.rotation.reshape(-1).tolist()), cam.focal_x, cam.focal_y, cam.zFar, cam.zNear,
        fr.ctr.data_ptr(), fr.ws.data_ptr(), fr.ws.numel(), scratch.data_ptr(), scratch.numel(), tu.data_ptr(),
        fr.vu.data_ptr(), ts.data_ptr(), fr.vs.data_ptr(), fr.cap, fr.xy.data_ptr(), fr.rgbd.data_ptr(),
        fr.con.data_ptr(), fr.ranges.data_ptr(), f3(0.0, 0.0, 0.0), out.data_ptr(),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    check(st, "forward_depth_first")
    n = ctypes.c_int32(0)
    check(lib().gsr_read_status(ctypes.c_void_p(fr.ws.data_ptr()), ctypes.c_void_p(fr.ctr.data_ptr()), fr.cap,
                                ctypes.byref(n), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
          "read_status")
    M = n.value
    return out, M, ts[:M].cpu().numpy().view(np.uint32).copy(), fr.vs[:M].cpu().numpy().view(np.uint32).copy()


@pytest.mark.parametrize("name,raw,spec", _cases(), ids=[c[0] for c in _cases()])
def test_depth_first_quads_equal_single_pass_quads(cuda_device, name, raw, spec):
    """The depth-first forward with quad keys: the same quad pairs as the
    single-pass quad emission (expanded to exactly the per-tile triples), in
    quad order, and the per-tile pipeline's image."""
    scene = Scene.from_raw(raw, cuda_device)
    cam = Camera.from_spec(spec)
    fr = _Frame(scene, 8_000_000, cuda_device)
    scratch = torch.zeros(lib().gsr_depth_first_scratch_size(scene.num_vertex), dtype=torch.int8, device=cuda_device)
    gx = (cam.width + 15) // 16
    img_t, kt, vt, _ = fr.forward(cam, R.RENDER_PERSISTENT_FUSED)
    img_t = img_t.clone()
    _, kq, _, _ = fr.forward(cam, R.RENDER_PERSISTENT_FUSED | QUAD)
    # stale pairs in the buffers must not matter: fill them first
    fr.ku.fill_(-7)
    fr.ks.fill_(-7)
    fr.vu.fill_(-7)
    fr.vs.fill_(-7)
    img_d, M, tiles, vals = _depth_first(fr, cam, R.RENDER_PERSISTENT_FUSED | QUAD, scratch)
    assert M == len(kq), (M, len(kq))
    assert torch.equal(img_d, img_t), int((img_d != img_t).sum())
    assert np.all(np.diff(tiles.astype(np.int64)) >= 0)
    depth = (kt & np.uint64(0xFFFFFFFF)).astype(np.int64)
    by_gid = dict(zip(vt.tolist(), depth.tolist()))
    keys = (tiles.astype(np.uint64) << np.uint64(32)) | np.array(
        [by_gid[int(v & ((1 << 28) - 1))] for v in vals], dtype=np.uint64)
    assert np.array_equal(_sorted_rows(_expand_quads(keys, vals, gx)), _sorted_rows(_per_tile(kt, vt)))


def test_batched_quads_equal_single_view_per_tile_images(cuda_device):
    """Several views through the batcher with quad keys, and the emission
    thresholds lowered so that most rectangles take the large-Gaussian queue
    and the queue overflows into the in-place sweep."""
    raws = [scenes.scene_clustered(3_000_000, seed=1),
            scenes.scene_clustered(50_000, seed=33),
            scenes.subsample(scenes.scene_plain_small(), 30_000, seed=1)]
    scs = [Scene.from_raw(r, cuda_device) for r in raws]
    f = scenes.focal_for
    views = [(0, scenes.camera_front(1920, 1080, 1400.0)),
             (1, scenes.orbit_camera(8.0, 0.7, 0.3, 1280, 720, f(1280))),
             (2, scenes.camera_front(800, 600, 600.0)),
             (0, scenes.orbit_camera(9.0, 2.0, -0.2, 1000, 584, f(1000))),
             (0, scenes.orbit_camera(7.0, 3.5, 0.1, 1920, 1080, f(1920)))]
    bg = [0.1, 0.2, 0.3]
    singles = []
    for si, spec in views:
        fr = _Frame(scs[si], 16_000_000, cuda_device)
        img, _, _, _ = fr.forward(Camera.from_spec(spec), R.RENDER_PERSISTENT_FUSED, bg)
        singles.append(img.clone())
        del fr
    for thresholds in ((32, 2048), (2, 4)):
        b = Batcher(8, 24_000_000, sum(scs[si].num_vertex for si, _ in views), 40_000, cuda_device)
        b.set_thresholds(*thresholds)
        vs = [View(si, Camera.from_spec(spec), bg) for si, spec in views]
        b.render(scs, vs, variant=R.RENDER_PERSISTENT_FUSED | QUAD, half=True, use_graph=False)
        b.finish()
        for (si, spec), v, want in zip(views, vs, singles):
            assert torch.equal(v.out, want), (thresholds, spec.width, int((v.out != want).sum()))
        if thresholds == (2, 4):
            # word 3 of the workspace header counts the rectangles sent to
            # the warp-swept region of the large-Gaussian queue (2^20 - 2^15
            # slots; huge ones that found the CTA-swept region full come here
            # too): past it, the in-place sweep ran
            words = torch.as_tensor(_DevWords(lib().gsr_batcher_status(b._h), 4), device=cuda_device).cpu()
            assert int(words[3]) > (1 << 20) - (1 << 15), words
        b.close()


def test_quad_image_equals_reference_e2e(cuda_device):
    from oracle import refkernels as RK

    if not RK.available():
        pytest.skip("reference kernels not built")
    raw = scenes.subsample(scenes.scene_clustered(600_000, seed=1), 200_000, seed=6)
    spec = scenes.orbit_camera(8.0, 1.3, 0.25, 1920, 1080, scenes.focal_for(1920))
    scene = Scene.from_raw(raw, cuda_device)
    fr = _Frame(scene, 8_000_000, cuda_device)
    img, _, _, _ = fr.forward(Camera.from_spec(spec), R.RENDER_PERSISTENT_FUSED | QUAD)
    pipe = RK.Pipeline(scene, spec, 16_000_000)
    pipe.forward()
    torch.cuda.synchronize()
    assert torch.equal(img, pipe.out), int((img != pipe.out).sum())


def test_quad_rejects_other_tile_shapes(cuda_device):
    raw = scenes.subsample(scenes.scene_plain_small(), 5_000, seed=1)
    scene = Scene.from_raw(raw, cuda_device)
    cam = Camera.from_spec(scenes.camera_front(320, 240, 240.0))
    b = Batcher(2, 100_000, scene.num_vertex, 4096, cuda_device)
    with pytest.raises(R.GsrError):
        b.render([scene], [View(0, cam)], variant=R.RENDER_PERSISTENT_FUSED | QUAD, block_x=32, block_y=32,
                 use_graph=False)
    b.close()
