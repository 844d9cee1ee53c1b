"""Drop-in ``Scene`` / ``Camera`` / ``Rasterizer`` (the reference's ``example.py``).

``Rasterizer.forward(scene, camera, bg_color, block_x=16, block_y=16,
render_variant="default", measure_preprocess=False, measure_sort=False,
measure_render=False, return_stats=False, use_es="auto")`` keeps the
reference's signature, variant names and return shapes
(``example.py:293-824``).  Buffers are allocated once in the constructor from
``MAX_NUM_RENDERED`` / ``MAX_NUM_TILES`` as the reference does, minus the
ablation-only buffers (compact features, top-k caches, tile descriptors),
which are allocated lazily on first use.
"""
from __future__ import annotations

import json
import os

import numpy as np
import torch

from . import ops


class Scene:
    """Resident Gaussian scene (``example.py:12-30``)."""

    def __init__(self, device):
        self.device = torch.device(device)
        self.num_vertex = 0
        self.position = None
        self.shs = None
        self.shs_half = None
        self.opacity = None
        self.cov3d = None

    def loadPly(self, scene_path):
        self.num_vertex, self.position, self.shs, self.opacity, self.cov3d = ops.loadPly(scene_path)
        self.position = self.position.to(self.device)
        self.shs = self.shs.to(self.device)
        self.shs_half = self.shs.half()
        self.opacity = self.opacity.to(self.device)
        self.cov3d = self.cov3d.to(self.device)

    @classmethod
    def from_raw(cls, raw, device="cuda", keep_fp32_sh: bool = True):
        """Build from raw INRIA parameters (a :class:`scenes.RawScene`); the
        parameter transform runs on the GPU (``gsr_scene_prepare``)."""
        s = cls(device)
        dev = s.device
        s.num_vertex = raw.num
        s.position = torch.from_numpy(np.ascontiguousarray(raw.means, np.float32)).to(dev)
        shs = torch.from_numpy(np.ascontiguousarray(raw.shs, np.float32).reshape(raw.num, 48)).to(dev)
        s.shs_half = shs.half()
        s.shs = shs if keep_fp32_sh else None
        s.opacity, s.cov3d = ops.prepare_scene(
            torch.from_numpy(np.ascontiguousarray(raw.log_scales, np.float32)).to(dev),
            torch.from_numpy(np.ascontiguousarray(raw.quats, np.float32)).to(dev),
            torch.from_numpy(np.ascontiguousarray(raw.opacity_logits, np.float32)).to(dev))
        return s

    def device_bytes(self) -> int:
        n = 0
        for t in (self.position, self.shs, self.shs_half, self.opacity, self.cov3d):
            if t is not None:
                n += t.numel() * t.element_size()
        return n


class Camera:
    """Pinhole camera from a ``cameras.json`` entry (``example.py:33-44``)."""

    def __init__(self, camera_json):
        self.id = camera_json.get("id", 0)
        self.img_name = camera_json.get("img_name", "")
        self.width = int(camera_json["width"])
        self.height = int(camera_json["height"])
        self.position = torch.tensor(camera_json["position"], dtype=torch.float32)
        self.rotation = torch.tensor(camera_json["rotation"], dtype=torch.float32)
        self.focal_x = float(camera_json["fx"])
        self.focal_y = float(camera_json["fy"])
        self.zFar = 100.0
        self.zNear = 0.01

    @classmethod
    def from_spec(cls, spec):
        return cls(spec.to_json())


E2E = "preranges_smem_persistent_lite_e2e"
E2E_PRERANGES = "preranges_smem_persistent_lite_e2e_preranges"
LITE = "preranges_smem_persistent_lite"


class Rasterizer:
    AUTO_RENDER_CANDIDATES = ((16, 16, "default"), (32, 16, "split"))

    def __init__(self, scene, MAX_NUM_RENDERED, MAX_NUM_TILES, enable_es=True):
        dev = scene.device
        self.device = dev
        self.MAX_NUM_RENDERED = int(MAX_NUM_RENDERED)
        self.MAX_NUM_TILES = int(MAX_NUM_TILES)
        n = self.MAX_NUM_RENDERED
        self.gaussian_keys_unsorted = torch.zeros(n, device=dev, dtype=torch.int64)
        self.gaussian_values_unsorted = torch.zeros(n, device=dev, dtype=torch.int32)
        self.gaussian_keys_sorted = torch.zeros(n, device=dev, dtype=torch.int64)
        self.gaussian_values_sorted = torch.zeros(n, device=dev, dtype=torch.int32)
        self.SORT_BUFFER_SIZE = ops.get_sort_buffer_size(n)
        self.list_sorting_space = torch.zeros(self.SORT_BUFFER_SIZE, device=dev, dtype=torch.int8)
        self.curr_offset = torch.zeros(1, device=dev, dtype=torch.int32)
        P = max(1, scene.num_vertex)
        self.points_xy = torch.zeros((P, 2), device=dev, dtype=torch.float32)
        self.rgb_depth = torch.zeros((P, 4), device=dev, dtype=torch.float32)
        self.conic_opacity = torch.zeros((P, 4), device=dev, dtype=torch.float32)
        self.tile_ranges_buf = torch.zeros((self.MAX_NUM_TILES, 2), device=dev, dtype=torch.int32)
        self.enable_es = enable_es
        # adaptive choice of the depth-first ("early sorting") pipeline, with
        # the reference's thresholds and environment overrides (example.py:70-90)
        self._es_threshold_M = int(os.environ.get("POLYSPLAT_ES_THRESHOLD_M", "5000000"))
        self._es_threshold_N_firstcall = int(os.environ.get("POLYSPLAT_ES_THRESHOLD_N", "3000000"))
        self._es_ratio_thresh = float(os.environ.get("POLYSPLAT_ES_RATIO_THRESH", "0.7"))
        self._es_firstcall_huge_P_guard = int(os.environ.get("POLYSPLAT_ES_FIRSTCALL_HUGE_P", "30000000"))
        self._es_force_two_pass = os.environ.get("POLYSPLAT_ES_FORCE_TWO_PASS", "0") not in ("0", "", "false",
                                                                                          "False")
        self._df_scratch = None
        self._compact = None
        self._out_color = None
        self._auto_render_choice = None
        self._es_last_M = None

    # -- buffers ------------------------------------------------------------------
    def _get_out_color(self, height, width, device):
        if self._out_color is None or self._out_color.shape[0] != height or self._out_color.shape[1] != width:
            self._out_color = torch.zeros((height, width, 3), device=device, dtype=torch.uint8)
        return self._out_color

    def _compact_buffers(self):
        if self._compact is None:
            n, dev = self.MAX_NUM_RENDERED, self.device
            self._compact = (torch.zeros((n, 2), device=dev, dtype=torch.float32),
                             torch.zeros((n, 4), device=dev, dtype=torch.float32),
                             torch.zeros((n, 4), device=dev, dtype=torch.float32),
                             torch.arange(n, device=dev, dtype=torch.int32))
        return self._compact

    def _check_tiles(self, camera, bx, by):
        t = ((camera.width + bx - 1) // bx) * ((camera.height + by - 1) // by)
        if t > self.MAX_NUM_TILES:
            raise ValueError("image needs %d tiles, MAX_NUM_TILES is %d" % (t, self.MAX_NUM_TILES))

    # -- autotune of the tile shape (example.py:199-231) ----------------------------
    def _autotune_render_config(self, scene, camera, bg_color, measure_runs=2):
        best, best_ms = None, None
        for bx, by, variant in self.AUTO_RENDER_CANDIDATES:
            self.forward(scene, camera, bg_color, block_x=bx, block_y=by, render_variant=variant)
            total = 0.0
            for _ in range(measure_runs):
                _, st = self.forward(scene, camera, bg_color, block_x=bx, block_y=by, render_variant=variant,
                                     measure_preprocess=True, measure_sort=True, measure_render=True,
                                     return_stats=True)
                total += st["preprocess_ms"] + st["sort_ms"] + st["render_ms"]
            if best_ms is None or total < best_ms:
                best, best_ms = (bx, by, variant), total
        self._auto_render_choice = best
        return best

    # -- depth-first ("early sorting") routing (example.py:246-291) ------------------
    def _decide_use_es(self, scene, use_es, render_variant):
        """The reference's rule: never for the fused E2E variants; True/False
        as given; "auto" takes it when the last frame's key count M is large
        in absolute terms and relative to P, or on a first call when P is
        large but below the huge-scene guard."""
        if not self.enable_es or render_variant in (E2E, E2E_PRERANGES):
            return False
        if use_es is True or use_es is False:
            return use_es
        if self._es_force_two_pass:
            return True
        P = scene.num_vertex
        if self._es_last_M is not None:
            M = self._es_last_M
            return M > self._es_threshold_M and M > self._es_ratio_thresh * P
        if P > self._es_firstcall_huge_P_guard:
            return False
        return P > self._es_threshold_N_firstcall

    @staticmethod
    def _df_variant(render_variant):
        from . import _lib as R
        if render_variant.endswith("_dt"):
            return R.RENDER_DT
        if render_variant == LITE or render_variant.startswith("preranges_smem_persistent"):
            return R.RENDER_PERSISTENT_RANGES
        if render_variant.startswith("preranges") or render_variant.startswith("reordered"):
            return R.RENDER_RANGES_CADENCE2
        return R.RENDER_DEFAULT

    def _forward_depth_first(self, scene, args_cam, render_variant, bg_color, out):
        n = self.MAX_NUM_RENDERED
        if self._df_scratch is None:
            self._df_scratch = torch.zeros(ops.depth_first_scratch_size(scene.num_vertex), device=self.device,
                                           dtype=torch.int8)
        half = render_variant.startswith("preranges_smem")
        # 32-bit tile ids live in the front half of the 64-bit key buffers
        tiles_u = self.gaussian_keys_unsorted.view(torch.int32)[:n]
        tiles_s = self.gaussian_keys_sorted.view(torch.int32)[:n]
        return ops.forward_depth_first(self._df_variant(render_variant), half, scene.position,
                                       scene.shs_half if half else scene.shs, scene.opacity, scene.cov3d,
                                       *args_cam, self.curr_offset, self.list_sorting_space, self._df_scratch,
                                       tiles_u, self.gaussian_values_unsorted, tiles_s, self.gaussian_values_sorted,
                                       self.points_xy, self.rgb_depth, self.conic_opacity, self.tile_ranges_buf,
                                       bg_color, out)

    # -- forward --------------------------------------------------------------------
    def forward(self, scene, camera, bg_color, block_x=16, block_y=16, render_variant="default",
                measure_preprocess=False, measure_sort=False, measure_render=False, return_stats=False,
                use_es="auto"):
        requested = render_variant
        if render_variant == "auto":
            if self._auto_render_choice is None:
                self._autotune_render_config(scene, camera, bg_color)
            block_x, block_y, render_variant = self._auto_render_choice
        measuring = measure_preprocess or measure_sort or measure_render
        if render_variant in (E2E, E2E_PRERANGES) and measuring:
            render_variant = LITE  # E2E paths expose no per-stage events (example.py:364-368)
        self._check_tiles(camera, block_x, block_y)
        out = self._get_out_color(camera.height, camera.width, scene.device)
        args_cam = (camera.width, camera.height, block_x, block_y, camera.position, camera.rotation,
                    camera.focal_x, camera.focal_y, camera.zFar, camera.zNear)
        bufs = (self.gaussian_keys_unsorted, self.gaussian_values_unsorted, self.gaussian_keys_sorted,
                self.gaussian_values_sorted)
        feats = (self.points_xy, self.rgb_depth, self.conic_opacity)

        fused = None
        used_es = False
        if not measuring and self._decide_use_es(scene, use_es, render_variant):
            used_es = True
            fused = lambda: self._forward_depth_first(scene, args_cam, render_variant, bg_color, out)
        elif not measuring:
            if render_variant == E2E:
                fused = lambda: ops.forward_fused_e2e(scene.position, scene.shs_half, scene.opacity, scene.cov3d,
                                                      *args_cam, self.curr_offset, self.list_sorting_space, *bufs,
                                                      *feats, bg_color, out)
            elif render_variant == E2E_PRERANGES:
                fused = lambda: ops.forward_fused_e2e_preranges(
                    scene.position, scene.shs_half, scene.opacity, scene.cov3d, *args_cam, self.curr_offset,
                    self.list_sorting_space, *bufs, *feats, self.tile_ranges_buf, bg_color, out)
            elif render_variant in ("default", "unroll2", "split"):
                fused = lambda: ops.forward_fused(scene.position, scene.shs, scene.opacity, scene.cov3d,
                                                  *args_cam[:4], *args_cam[4:], render_variant, self.curr_offset,
                                                  self.list_sorting_space, *bufs, *feats, bg_color, out)
        if fused is not None:
            num = fused()
            self._es_last_M = num
            if return_stats:
                return out, self._stats(requested, render_variant, block_x, block_y, num, None, None, None,
                                        used_es)
            return out

        # ---- per-stage path (example.py:481-781) ----
        half = render_variant.startswith("preranges_smem")
        ev = {}

        def mark(name):
            if measuring:
                e = torch.cuda.Event(enable_timing=True)
                e.record()
                ev[name] = e

        self.curr_offset.zero_()
        mark("pre0")
        if half:
            ops.preprocess_half_sh(scene.position, scene.shs_half, scene.opacity, scene.cov3d, *args_cam, *feats,
                                   self.gaussian_keys_unsorted, self.gaussian_values_unsorted, self.curr_offset)
        else:
            ops.preprocess(scene.position, scene.shs, scene.opacity, scene.cov3d, *args_cam, *feats,
                           self.gaussian_keys_unsorted, self.gaussian_values_unsorted, self.curr_offset)
        mark("pre1")
        num = int(self.curr_offset.cpu()[0])
        if num > self.MAX_NUM_RENDERED:
            raise RuntimeError("Too many k-v pairs! (%d > %d)" % (num, self.MAX_NUM_RENDERED))
        mark("sort0")
        ops.sort_gaussian(num, camera.width, camera.height, block_x, block_y, self.list_sorting_space, *bufs)
        mark("sort1")
        W, H = camera.width, camera.height
        xy, rgbd, con = feats
        vals = self.gaussian_values_sorted
        if render_variant in ("gathered", "gathered_unroll2", "preranges_gathered"):
            cxy, crgbd, ccon, ident = self._compact_buffers()
            ops.gather_features(num, vals, xy, rgbd, con, cxy, crgbd, ccon)
            xy, rgbd, con, vals = cxy, crgbd, ccon, ident
        needs_ranges = render_variant.startswith("preranges") and render_variant not in ("preranges_smem_v2",)
        if render_variant == "preranges_scan":
            ops.precompute_tile_ranges_scan(num, W, H, block_x, block_y, self.gaussian_keys_sorted,
                                            self.tile_ranges_buf)
        elif needs_ranges or render_variant.startswith("reordered"):
            ops.precompute_tile_ranges(num, W, H, block_x, block_y, self.gaussian_keys_sorted, self.tile_ranges_buf)
        mark("ren0")
        self._render_stage(render_variant, num, W, H, block_x, block_y, xy, rgbd, con, vals, bg_color, out)
        mark("ren1")
        self._es_last_M = num
        pre_ms = sort_ms = ren_ms = None
        if measuring:
            ev["ren1"].synchronize()
            if measure_preprocess:
                pre_ms = ev["pre0"].elapsed_time(ev["pre1"])
            if measure_sort:
                sort_ms = ev["sort0"].elapsed_time(ev["sort1"])
            if measure_render:
                ren_ms = ev["ren0"].elapsed_time(ev["ren1"])
        if return_stats:
            return out, self._stats(requested, render_variant, block_x, block_y, num, pre_ms, sort_ms, ren_ms, False)
        ret = [out]
        if measure_preprocess:
            ret.append(pre_ms)
        if measure_sort:
            ret.append(sort_ms)
        if measure_render:
            ret.append(ren_ms)
        return out if len(ret) == 1 else tuple(ret)

    def _render_stage(self, variant, num, W, H, bx, by, xy, rgbd, con, vals, bg, out):
        ks, rb = self.gaussian_keys_sorted, self.tile_ranges_buf
        if variant == LITE or variant.startswith("preranges_smem_persistent"):
            if variant.endswith("_dt"):
                ops.render_16x16_preranges_smem_persistent_lite_dt(num, W, H, xy, rgbd, con, vals, rb, bg, out)
            else:
                ops.render_16x16_preranges_smem_persistent_lite(num, W, H, xy, rgbd, con, vals, rb, bg, out)
        elif variant in ("preranges_smem", "preranges_naive"):
            ops.render_16x16_preranges_smem(num, W, H, xy, rgbd, con, vals, rb, bg, out)
        elif variant == "preranges_smem_v2":
            ops.render_16x16_preranges_smem_v2(num, W, H, xy, rgbd, con, ks, vals, bg, out)
        elif variant.startswith("preranges") or variant.startswith("reordered"):
            ops.render_16x16_preranges(num, W, H, xy, rgbd, con, vals, rb, bg, out)
        else:
            from ._lib import RENDER_DEFAULT
            ops._render(RENDER_DEFAULT, num, W, H, xy, rgbd, con, ks, vals, None, bg, out, bx, by)

    @staticmethod
    def _stats(requested, variant, bx, by, num, pre, srt, ren, used_es):
        return {"requested_render_variant": requested, "render_variant": variant, "resolved_block_x": bx,
                "resolved_block_y": by, "num_rendered": num, "preprocess_ms": pre, "sort_ms": srt,
                "render_ms": ren, "used_es": used_es}


def savePpm(image, path):
    image = image.cpu()
    assert image.dim() >= 3 and image.size(2) == 3
    with open(path, "wb") as f:
        f.write(b"P6\n" + f"{image.size(1)} {image.size(0)}\n255\n".encode() + image.numpy().tobytes())
