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

``render_views`` renders several cameras of one size in one pass
(``gsr_train_forward_views`` / ``gsr_train_backward_views``): one preprocess
launch over every view, one sort of all views' keys, one render and one
render backward over every view's tiles, and one adjoint launch per 16 views
that sums the views' gradients per Gaussian, so the parameters are read and
their gradients written once per pass instead of once per camera.  Its sort
takes quad keys by default (one key per 2x2 group of tiles, the same images),
and ``stacked=True`` returns the views as one [views, H, W, 3] tensor so a
loss over all of them is one operation.
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


def _views_cam_args(cams: Sequence[Camera]):
    pos = [float(v) for c in cams for v in c.position.reshape(-1).tolist()]
    rot = [float(v) for c in cams for v in c.rotation.reshape(-1).tolist()]
    intr = [float(v) for c in cams for v in (c.focal_x, c.focal_y, c.zFar, c.zNear)]
    return (ctypes.c_float * len(pos))(*pos), (ctypes.c_float * len(rot))(*rot), (ctypes.c_float * len(intr))(*intr)


class _RenderViewsFn(torch.autograd.Function):
    """All views in one pass (gsr_train_forward_views / gsr_train_backward_views)."""

    @staticmethod
    def forward(ctx, means, log_scales, quats, logits, shs, cams, bg, key_capacity, quad_keys=True):
        dev = means.device
        P, V = means.shape[0], len(cams)
        flags = R.QUAD_KEYS if quad_keys else 0
        W, H = cams[0].width, cams[0].height
        tiles = ((W + 15) // 16) * ((H + 15) // 16)
        pos, rot, intr = _views_cam_args(cams)
        bgc = (ctypes.c_float * 3)(*[float(v) for v in bg])
        params = [t.detach().contiguous().float() for t in (means, log_scales, quats, logits, shs.reshape(P, 48))]
        stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        scratch = torch.empty(lib().gsr_train_views_scratch_bytes(V), dtype=torch.int8, device=dev)
        cap = int(key_capacity)
        while True:
            b = dict(
                opacity=torch.empty(P, device=dev), cov3d=torch.empty((P, 6), device=dev),
                count=torch.zeros(1, dtype=torch.int32, device=dev),
                ws=torch.empty(get_sort_buffer_size(cap), dtype=torch.int8, device=dev),
                ku=torch.empty(cap, dtype=torch.int64, device=dev), vu=torch.empty(cap, dtype=torch.int32, device=dev),
                ks=torch.empty(cap, dtype=torch.int64, device=dev), vs=torch.empty(cap, dtype=torch.int32, device=dev),
                xy=torch.empty((V * P, 2), device=dev), rgbd=torch.empty((V * P, 4), device=dev),
                con=torch.empty((V * P, 4), device=dev), ranges=torch.empty((V * tiles, 2), dtype=torch.int32, device=dev),
                n_tile=torch.empty(V * tiles, dtype=torch.int32, device=dev), T=torch.empty((V, H, W), device=dev),
                image=torch.empty((V, H, W, 3), device=dev))
            check(lib().gsr_train_forward_views(
                P, *[_p(t) for t in params], V, W, H, pos, rot, intr, bgc, _p(b["opacity"]), _p(b["cov3d"]),
                _p(scratch), scratch.numel(), _p(b["count"]), _p(b["ws"]), b["ws"].numel(), _p(b["ku"]), _p(b["vu"]),
                _p(b["ks"]), _p(b["vs"]), cap, _p(b["xy"]), _p(b["rgbd"]), _p(b["con"]), _p(b["ranges"]),
                _p(b["n_tile"]), _p(b["T"]), _p(b["image"]), flags, stream), "train_forward_views")
            n = ctypes.c_int32(0)
            st = lib().gsr_read_status(_p(b["ws"]), _p(b["count"]), cap, ctypes.byref(n), stream)
            if st == R.GSR_OVERFLOW:
                cap = max(2 * cap, int(n.value * 1.25))
                if cap >= 1 << 30:
                    raise R.GsrError(st, "train_forward_views: more keys than one sort takes", n.value)
                continue
            check(st, "train_forward_views", n.value)
            break
        for k in ("ku", "ks", "ws", "opacity", "cov3d"):
            del b[k]
        ctx.b, ctx.cams, ctx.bg, ctx.cap, ctx.flags = b, list(cams), [float(v) for v in bg], cap, flags
        ctx.save_for_backward(*params)
        ctx.num_rendered = n.value
        return b["image"]

    @staticmethod
    def backward(ctx, grad_image):
        means, log_scales, quats, logits, shs = ctx.saved_tensors
        b, cams = ctx.b, ctx.cams
        dev = means.device
        P, V = means.shape[0], len(cams)
        g = grad_image.contiguous().float()
        pos, rot, intr = _views_cam_args(cams)
        bgc = (ctypes.c_float * 3)(*ctx.bg)
        gfeat = torch.empty((V * P, 12), device=dev)
        outs = [torch.empty_like(t) for t in (means, log_scales, quats, logits, shs)]
        stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        check(lib().gsr_train_backward_views(
            P, _p(means), _p(log_scales), _p(quats), _p(logits), _p(shs), V, cams[0].width, cams[0].height, pos, rot,
            intr, bgc, _p(b["count"]), ctx.cap, _p(b["vs"]), _p(b["ranges"]), _p(b["n_tile"]), _p(b["T"]),
            _p(b["xy"]), _p(b["rgbd"]), _p(b["con"]), _p(g), _p(gfeat), *[_p(t) for t in outs], 0, ctx.flags,
            stream), "train_backward_views")
        ctx.b = None
        gm, gls, gq, glg, gsh = outs
        return gm, gls, gq, glg, gsh, None, None, None, None


def render_views(means, log_scales, quats, logits, shs, cameras: Sequence[Camera], bg=(0.0, 0.0, 0.0),
                 key_capacity: int = 1 << 22, quad_keys: bool = True, stacked: bool = False):
    """One differentiable image per camera (gradients sum over views).

    Cameras of one size go through one pass over all views: one preprocess
    launch, one sort of every view's keys, one render and one render backward
    over every view's tiles, and one adjoint that sums the views' gradients
    per Gaussian (`key_capacity` is per view).  With `quad_keys` the sort
    takes one key per 2x2 group of tiles (the same images; fewer keys and
    tile bits).  Cameras of different sizes fall back to one pass per
    camera.  Returns a list of [H, W, 3] images, or with `stacked` (cameras
    of one size) one [views, H, W, 3] tensor, so that a loss over all views
    is one operation."""
    cams = list(cameras)
    same = all((c.width, c.height) == (cams[0].width, cams[0].height) for c in cams) if cams else True
    if stacked and not same:
        raise ValueError("render_views(stacked=True) needs cameras of one size")
    if not cams:
        return [] if not stacked else torch.empty((0, 0, 0, 3), device=means.device)
    if len(cams) == 1 or not same:
        imgs = [render(means, log_scales, quats, logits, shs, c, bg, key_capacity) for c in cams]
        return torch.stack(imgs) if stacked else imgs
    cap = min(int(key_capacity) * len(cams), (1 << 30) - 1)
    quad = bool(quad_keys) and means.shape[0] * len(cams) <= (1 << 28)
    out = _RenderViewsFn.apply(means, log_scales, quats, logits, shs.reshape(shs.shape[0], 48), cams, list(bg), cap,
                               quad)
    return out if stacked else list(out.unbind(0))
