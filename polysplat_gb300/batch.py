"""Batched forward: several views (of different scenes and resolutions)
rendered by one pass of the pipeline, optionally replayed from a CUDA graph.

No counterpart in the reference, which renders one view per call.  The
device work is the C ABI's ``gsr_batcher_*`` (``csrc/batch.cu``); this module
only packs the per-view descriptors.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import torch

from . import _lib as R
from ._lib import GsrError, check, lib


class SceneRef(ctypes.Structure):
    _fields_ = [("P", ctypes.c_int), ("pos", ctypes.c_void_p), ("shs", ctypes.c_void_p),
                ("opacity", ctypes.c_void_p), ("cov3d", ctypes.c_void_p)]


class ViewDesc(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_int), ("width", ctypes.c_int), ("height", ctypes.c_int),
                ("cam_pos", ctypes.c_float * 3), ("cam_rot", ctypes.c_float * 9), ("focal_x", ctypes.c_float),
                ("focal_y", ctypes.c_float), ("z_far", ctypes.c_float), ("z_near", ctypes.c_float),
                ("bg", ctypes.c_float * 3), ("out", ctypes.c_void_p)]


class View:
    """One view of a batch: a scene index, a Camera, a background and the
    caller's output image (CUDA uint8 [H, W, 3])."""

    def __init__(self, scene: int, camera, bg=(0.0, 0.0, 0.0), out: Optional[torch.Tensor] = None):
        self.scene = int(scene)
        self.camera = camera
        self.bg = [float(x) for x in (bg.tolist() if isinstance(bg, torch.Tensor) else bg)]
        self.out = out


class Batcher:
    """Owns the device buffers of batched frames (allocated once)."""

    def __init__(self, max_views: int, key_capacity: int, max_gaussians: int, max_tiles: int, device=None):
        self.device = torch.device(device or "cuda")
        with torch.cuda.device(self.device):
            self._h = lib().gsr_batcher_create(int(max_views), int(key_capacity), int(max_gaussians), int(max_tiles))
        if not self._h:
            raise GsrError(R.GSR_INVALID_ARG, "gsr_batcher_create (sizes or device memory)")
        self.max_views, self.key_capacity = int(max_views), int(key_capacity)
        self.max_gaussians, self.max_tiles = int(max_gaussians), int(max_tiles)
        self._scenes_keep = None

    @staticmethod
    def device_bytes(max_views, key_capacity, max_gaussians, max_tiles) -> int:
        return int(lib().gsr_batcher_device_bytes(int(max_views), int(key_capacity), int(max_gaussians),
                                                  int(max_tiles)))

    def close(self):
        if getattr(self, "_h", None):
            lib().gsr_batcher_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_thresholds(self, massive_area: int, huge_area: int) -> None:
        """Dispatch thresholds of the tile-key emission (tiles of a rectangle)."""
        check(lib().gsr_batcher_set_thresholds(self._h, int(massive_area), int(huge_area)), "batcher_set_thresholds")

    @property
    def graphs(self) -> int:
        return int(lib().gsr_batcher_graphs(self._h))

    def counter_ptr(self) -> int:
        return int(lib().gsr_batcher_counter(self._h))

    def render(self, scenes: Sequence, views: Sequence[View], variant: int = R.RENDER_PERSISTENT_FUSED,
               half: bool = True, block_x: int = 16, block_y: int = 16, use_graph: bool = True,
               stream: Optional[torch.cuda.Stream] = None) -> None:
        """Enqueue one batch (asynchronous).  Allocates each view's output
        image if it has none."""
        n = len(views)
        sc = (SceneRef * len(scenes))()
        for i, s in enumerate(scenes):
            shs = s.shs_half if half else s.shs
            sc[i] = SceneRef(int(s.num_vertex), s.position.data_ptr(), shs.data_ptr(), s.opacity.data_ptr(),
                             s.cov3d.data_ptr())
        vd = (ViewDesc * n)()
        for i, v in enumerate(views):
            c = v.camera
            if v.out is None:
                v.out = torch.empty((c.height, c.width, 3), dtype=torch.uint8, device=self.device)
            d = vd[i]
            d.scene, d.width, d.height = v.scene, c.width, c.height
            d.cam_pos[:] = [float(x) for x in c.position.reshape(-1).tolist()]
            d.cam_rot[:] = [float(x) for x in c.rotation.reshape(-1).tolist()]
            d.focal_x, d.focal_y, d.z_far, d.z_near = c.focal_x, c.focal_y, c.zFar, c.zNear
            d.bg[:] = v.bg
            d.out = v.out.data_ptr()
        st = stream or torch.cuda.current_stream(self.device)
        self._scenes_keep = scenes  # the device pointers stay valid while the batch runs
        check(lib().gsr_batcher_render(self._h, int(variant), 1 if half else 0, int(block_x), int(block_y), sc,
                                       len(scenes), vd, n, 1 if use_graph else 0, ctypes.c_void_p(st.cuda_stream)),
              "batcher_render")

    def finish(self, stream: Optional[torch.cuda.Stream] = None) -> int:
        """Wait for the last batch; returns its key count (raises on overflow)."""
        st = stream or torch.cuda.current_stream(self.device)
        n = ctypes.c_int32(0)
        status = lib().gsr_batcher_finish(self._h, ctypes.byref(n), ctypes.c_void_p(st.cuda_stream))
        check(status, "batcher_finish", n.value)
        return n.value


def tiles_of(camera, bx=16, by=16) -> int:
    return ((camera.width + bx - 1) // bx) * ((camera.height + by - 1) // by)
