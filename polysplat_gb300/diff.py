"""Differentiable rendering: the forward rasterizer with a hand-written
backward behind ``torch.autograd.Function``.

No counterpart in the reference, which renders only.  The forward is the
library's pipeline (scene transform, preprocess with FP32 SH, radix sort,
tile ranges) with a render that writes a float image plus what the backward
replays: the sorted lists, each pixel's final transmittance and each tile's
number of blended Gaussians (csrc/render.cu ``k_render_train``).  The
backward walks every tile's list in reverse (``k_render_backward``) and
applies the per-Gaussian preprocess adjoint (``csrc/adjoint.h``) to reach the
raw parameters: means, log-scales, w-first quaternions, opacity logits and
SH coefficients.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import torch

from . import _lib as R
from ._lib import check, lib
from .ops import get_sort_buffer_size
from .rasterizer import Camera


def _p(t: torch.Tensor):
    return ctypes.c_void_p(t.data_ptr())


def _cam_args(cam: Camera):
    pos = (ctypes.c_float * 3)(*[float(v) for v in cam.position.reshape(-1).tolist()])
    rot = (ctypes.c_float * 9)(*[float(v) for v in cam.rotation.reshape(-1).tolist()])
    return pos, rot


class _RenderFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, means, log_scales, quats, logits, shs, cam, bg, key_capacity):
        dev = means.device
        P = means.shape[0]
        W, H = cam.width, cam.height
        tiles = ((W + 15) // 16) * ((H + 15) // 16)
        pos, rot = _cam_args(cam)
        bgc = (ctypes.c_float * 3)(*[float(v) for v in bg])
        params = [t.detach().contiguous().float() for t in (means, log_scales, quats, logits, shs.reshape(P, 48))]
        stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        cap = int(key_capacity)
        while True:
            b = dict(
                opacity=torch.empty(P, device=dev), cov3d=torch.empty((P, 6), device=dev),
                count=torch.zeros(1, dtype=torch.int32, device=dev),
                ws=torch.empty(get_sort_buffer_size(cap), dtype=torch.int8, device=dev),
                ku=torch.empty(cap, dtype=torch.int64, device=dev), vu=torch.empty(cap, dtype=torch.int32, device=dev),
                ks=torch.empty(cap, dtype=torch.int64, device=dev), vs=torch.empty(cap, dtype=torch.int32, device=dev),
                xy=torch.empty((P, 2), device=dev), rgbd=torch.empty((P, 4), device=dev),
                con=torch.empty((P, 4), device=dev), ranges=torch.empty((tiles, 2), dtype=torch.int32, device=dev),
                n_tile=torch.empty(tiles, dtype=torch.int32, device=dev), T=torch.empty((H, W), device=dev),
                image=torch.empty((H, W, 3), device=dev))
            check(lib().gsr_train_forward(
                P, *[_p(t) for t in params], W, H, pos, rot, cam.focal_x, cam.focal_y, cam.zFar, cam.zNear, bgc,
                _p(b["opacity"]), _p(b["cov3d"]), _p(b["count"]), _p(b["ws"]), b["ws"].numel(), _p(b["ku"]),
                _p(b["vu"]), _p(b["ks"]), _p(b["vs"]), cap, _p(b["xy"]), _p(b["rgbd"]), _p(b["con"]),
                _p(b["ranges"]), _p(b["n_tile"]), _p(b["T"]), _p(b["image"]), stream), "train_forward")
            n = ctypes.c_int32(0)
            st = lib().gsr_read_status(_p(b["ws"]), _p(b["count"]), cap, ctypes.byref(n), stream)
            if st == R.GSR_OVERFLOW:
                cap = max(2 * cap, int(n.value * 1.25))
                continue
            check(st, "train_forward", n.value)
            break
        for k in ("ku", "ks", "ws", "opacity", "cov3d"):
            del b[k]
        ctx.b, ctx.cam, ctx.bg, ctx.cap, ctx.P = b, cam, [float(v) for v in bg], cap, P
        ctx.save_for_backward(*params)
        ctx.num_rendered = n.value
        return b["image"]

    @staticmethod
    def backward(ctx, grad_image):
        means, log_scales, quats, logits, shs = ctx.saved_tensors
        b, cam, P = ctx.b, ctx.cam, ctx.P
        dev = means.device
        g = grad_image.contiguous().float()
        pos, rot = _cam_args(cam)
        bgc = (ctypes.c_float * 3)(*ctx.bg)
        gxy, gcon, grgb = (torch.empty((P, 2), device=dev), torch.empty((P, 4), device=dev),
                           torch.empty((P, 3), device=dev))
        outs = [torch.empty_like(t) for t in (means, log_scales, quats, logits, shs)]
        stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        check(lib().gsr_train_backward(
            P, _p(means), _p(log_scales), _p(quats), _p(logits), _p(shs), cam.width, cam.height, pos, rot,
            cam.focal_x, cam.focal_y, cam.zFar, cam.zNear, bgc, _p(b["count"]), ctx.cap, _p(b["vs"]),
            _p(b["ranges"]), _p(b["n_tile"]), _p(b["T"]), _p(b["xy"]), _p(b["rgbd"]), _p(b["con"]), _p(g), _p(gxy),
            _p(gcon), _p(grgb), *[_p(t) for t in outs], 0, stream), "train_backward")
        ctx.b = None
        gm, gls, gq, glg, gsh = outs
        return gm, gls, gq, glg, gsh, None, None, None


def render(means: torch.Tensor, log_scales: torch.Tensor, quats: torch.Tensor, logits: torch.Tensor,
           shs: torch.Tensor, camera: Camera, bg=(0.0, 0.0, 0.0), key_capacity: int = 1 << 22) -> torch.Tensor:
    """Differentiable float image [H, W, 3] of raw Gaussian parameters
    (means [P,3], log-scales [P,3], w-first quaternions [P,4], opacity logits
    [P], SH [P,16,3] or [P,48]) seen by `camera`."""
    shp = shs.shape
    out = _RenderFn.apply(means, log_scales, quats, logits, shs.reshape(shs.shape[0], 48), camera,
                          list(bg), key_capacity)
    return out


def render_views(means, log_scales, quats, logits, shs, cameras: Sequence[Camera], bg=(0.0, 0.0, 0.0),
                 key_capacity: int = 1 << 22):
    """One differentiable image per camera (gradients sum over views)."""
    return [render(means, log_scales, quats, logits, shs, c, bg, key_capacity) for c in cameras]
