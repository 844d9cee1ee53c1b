"""``polysplat.ops`` drop-in: the 43 operators of the reference's extension module.

Each function keeps the reference's name, positional argument order, dtypes
and in-place output convention (``csrc/pybind.cpp:1154-1372``) and forwards
to the gsr C ABI (``include/gsr.h``) on the current PyTorch CUDA stream.

Differences a caller can observe, all deliberate:

* every op runs on ``torch.cuda.current_stream()`` instead of the legacy
  default stream;
* key-buffer overflow raises :class:`GsrError` (status OVERFLOW with the true
  count) instead of writing past the buffer (the reference does not check,
  ``csrc/pybind.cpp:1124-1134``);
* ``get_sort_buffer_size(n)`` returns the size of this library's workspace
  (radix-sort ping-pong buffers, look-back state, tile queue and status word);
* the ES ("early sorting") helpers fill the reference's buffers with the
  reference's meanings; their scan scratch is this library's (see
  ``get_es_scan_buffer_size``) and the sort scratch is the workspace;
* the tile-reordering helpers are provided for API completeness; renders that
  take tile orders produce the same image as the plain persistent render
  because tile order never changes a tile's result.
"""
from __future__ import annotations

import ctypes
from typing import Dict, Tuple

import numpy as np
import torch

from . import _lib
from ._lib import GsrError, check, lib

__all__ = [
    "loadPly", "preprocess", "preprocess_half_sh", "preprocess_es_pass_a", "preprocess_es_pass_a_half_sh",
    "preprocess_es_pass_b", "es_depth_sort_and_scan", "es_tile_sort", "get_es_scan_buffer_size",
    "sort_gaussian", "get_sort_buffer_size", "gather_features", "render_16x16", "render_16x16_preranges",
    "render_16x16_preranges_smem", "render_16x16_preranges_smem_persistent",
    "render_16x16_preranges_smem_persistent_lite", "render_16x16_preranges_smem_persistent_lite_dt",
    "render_16x16_preranges_naive", "render_16x16_preranges_smem_v2", "render_16x16_topk_smem",
    "render_16x16_topk_smem_persistent", "render_16x16_topk_smem_persistent_v2", "precompute_tile_ranges",
    "precompute_tile_ranges_scan", "compute_tile_order", "get_tile_order_sort_temp_size",
    "render_16x16_reordered", "compute_tile_order_packed", "compute_tile_order_packed_morton",
    "render_16x16_reordered_v2", "render_16x16_reordered_persistent", "render_16x16_unroll2",
    "render_16x16_split", "render_24x16_split", "render_32x16", "render_32x16_split", "render_32x32",
    "sort_and_render", "forward_fused", "render_16x16_preranges_smem_persistent_lite_fused",
    "forward_fused_e2e", "forward_fused_e2e_preranges",
]

# ---------------------------------------------------------------------------
# helpers


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


def _dev(t: torch.Tensor, what: str, dtype=None) -> torch.Tensor:
    if not isinstance(t, torch.Tensor):
        raise TypeError("%s must be a torch.Tensor" % what)
    if not t.is_cuda:
        raise ValueError("%s must be a CUDA tensor" % what)
    if dtype is not None and t.dtype != dtype:
        raise TypeError("%s must be %s, got %s" % (what, dtype, t.dtype))
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous (outputs are written in place)" % what)
    return t


def _host_floats(t, n: int, what: str):
    """Camera position/rotation and background are read on the host."""
    if isinstance(t, torch.Tensor):
        vals = t.detach().to("cpu", torch.float32).reshape(-1).tolist()
    else:
        vals = [float(v) for v in np.asarray(t, dtype=np.float32).reshape(-1)]
    if len(vals) < n:
        raise ValueError("%s needs %d floats" % (what, n))
    return (ctypes.c_float * n)(*vals[:n])


def _stream(dev: torch.device) -> int:
    return torch.cuda.current_stream(dev).cuda_stream


_render_ws: Dict[Tuple[int, int], torch.Tensor] = {}


def _render_workspace(dev: torch.device) -> torch.Tensor:
    """Small per-(device, stream) workspace for render-only ops."""
    key = (dev.index if dev.index is not None else torch.cuda.current_device(), _stream(dev))
    ws = _render_ws.get(key)
    if ws is None:
        ws = torch.zeros(lib().gsr_render_workspace_size(), dtype=torch.uint8, device=dev)
        _render_ws[key] = ws
    return ws


def _tiles(W: int, H: int, bx: int, by: int) -> int:
    return ((W + bx - 1) // bx) * ((H + by - 1) // by)


def _read_status(ws: torch.Tensor, num_t, cap: int, where: str) -> int:
    n = ctypes.c_int32(0)
    st = lib().gsr_read_status(_ptr(ws), _ptr(num_t) if num_t is not None else None, cap, ctypes.byref(n),
                               _stream(ws.device))
    check(st, where, n.value)
    return n.value


# ---------------------------------------------------------------------------
# scene loading (csrc/pybind.cpp:12-120)

_PLY_FLOATS = 62


def read_ply_raw(path):
    """Parse an INRIA binary PLY (62 float32 per vertex) into raw numpy arrays:
    (num, pos [P,3], shs [P,16,3] interleaved, logits [P], log_scales [P,3],
    quats [P,4]).  SH are reordered from the file's channel-major f_rest to
    the interleaved layout (csrc/pybind.cpp:105-111)."""
    with open(path, "rb") as f:
        data = f.read()
    end = data.find(b"end_header")
    if end < 0:
        raise RuntimeError("Cannot find end of header")
    header = data[:end].decode("ascii", "replace").split()
    num = 0
    for i, tok in enumerate(header):
        if tok == "vertex" and i + 1 < len(header):
            num = int(header[i + 1])
    if num <= 0:
        raise RuntimeError("Vertex number is not positive")
    body_start = end + len(b"end_header")
    if data[body_start:body_start + 1] == b"\r":
        body_start += 1
    body_start += 1  # the newline after end_header
    need = num * _PLY_FLOATS * 4
    body = data[body_start:body_start + need]
    if len(body) < need:
        raise RuntimeError("PLY body is truncated (%d of %d bytes)" % (len(body), need))
    rec = np.frombuffer(body, dtype="<f4").reshape(num, _PLY_FLOATS)
    pos = np.ascontiguousarray(rec[:, 0:3])
    shs = np.empty((num, 16, 3), np.float32)
    shs[:, 0, :] = rec[:, 6:9]
    shs[:, 1:, :] = rec[:, 9:54].reshape(num, 3, 15).transpose(0, 2, 1)
    logits = np.ascontiguousarray(rec[:, 54])
    log_scales = np.ascontiguousarray(rec[:, 55:58])
    quats = np.ascontiguousarray(rec[:, 58:62])
    return num, pos, shs, logits, log_scales, quats


def loadPly(path, /):
    """Read an INRIA binary PLY -> (num, position, shs, opacity, cov3d) on the CPU.

    The parameter transform (sigmoid, exp, quaternion normalisation,
    Sigma = R S^2 R^T) runs as a CUDA kernel (``gsr_scene_prepare``) and the
    results are returned as CPU tensors, as the reference does."""
    num, pos, shs, logits, log_scales, quats = read_ply_raw(path)
    dev = torch.device("cuda", torch.cuda.current_device())
    op, cov = prepare_scene(torch.from_numpy(log_scales).to(dev), torch.from_numpy(quats).to(dev),
                            torch.from_numpy(logits).to(dev))
    return (num, torch.from_numpy(pos), torch.from_numpy(shs.reshape(num, 48)), op.cpu(), cov.cpu())


def prepare_scene(log_scales: torch.Tensor, quats: torch.Tensor, logits: torch.Tensor):
    """Raw parameters (device tensors) -> (opacity [P], cov3d [P,6]) on the device."""
    ls = _dev(log_scales.contiguous(), "log_scales", torch.float32)
    q = _dev(quats.contiguous(), "quats", torch.float32)
    lg = _dev(logits.contiguous(), "logits", torch.float32)
    P = lg.numel()
    op = torch.empty(P, dtype=torch.float32, device=lg.device)
    cov = torch.empty((P, 6), dtype=torch.float32, device=lg.device)
    check(lib().gsr_scene_prepare(P, _ptr(ls), _ptr(q), _ptr(lg), _ptr(op), _ptr(cov), _stream(lg.device)),
          "scene_prepare")
    return op, cov


# ---------------------------------------------------------------------------
# preprocess (csrc/pybind.cpp:122-181)

def _preprocess(half, orig_points, shs, opacities, cov3Ds, width, height, block_x, block_y, position, rotation,
                focal_x, focal_y, zFar, zNear, points_xy, rgb_depth, conic_opacity, keys_u, vals_u, curr_offset):
    pos = _dev(orig_points, "orig_points", torch.float32)
    sh = _dev(shs, "shs", torch.float16 if half else torch.float32)
    op = _dev(opacities, "opacities", torch.float32)
    cov = _dev(cov3Ds, "cov3Ds", torch.float32)
    for t, n in ((points_xy, "points_xy"), (rgb_depth, "rgb_depth"), (conic_opacity, "conic_opacity")):
        _dev(t, n, torch.float32)
    _dev(keys_u, "gaussian_keys_unsorted", torch.int64)
    _dev(vals_u, "gaussian_values_unsorted", torch.int32)
    _dev(curr_offset, "curr_offset", torch.int32)
    P = op.numel()
    cap = min(keys_u.numel(), vals_u.numel())
    ws = _render_workspace(op.device)
    st = lib().gsr_preprocess(P, _ptr(pos), _ptr(sh), 1 if half else 0, _ptr(op), _ptr(cov), int(width), int(height),
                              int(block_x), int(block_y), _host_floats(position, 3, "position"),
                              _host_floats(rotation, 9, "rotation"), float(focal_x), float(focal_y), float(zFar),
                              float(zNear), _ptr(points_xy), _ptr(rgb_depth), _ptr(conic_opacity), _ptr(keys_u),
                              _ptr(vals_u), cap, _ptr(curr_offset), _ptr(ws), ws.numel(), _stream(op.device))
    check(st, "preprocess")


def preprocess(orig_points, shs, opacities, cov3Ds, width, height, block_x, block_y, position, rotation,
               focal_x, focal_y, zFar, zNear, points_xy, rgb_depth, conic_opacity,
               gaussian_keys_unsorted, gaussian_values_unsorted, curr_offset, /):
    _preprocess(False, orig_points, shs, opacities, cov3Ds, width, height, block_x, block_y, position, rotation,
                focal_x, focal_y, zFar, zNear, points_xy, rgb_depth, conic_opacity, gaussian_keys_unsorted,
                gaussian_values_unsorted, curr_offset)


def preprocess_half_sh(orig_points, shs_half, opacities, cov3Ds, width, height, block_x, block_y, position,
                       rotation, focal_x, focal_y, zFar, zNear, points_xy, rgb_depth, conic_opacity,
                       gaussian_keys_unsorted, gaussian_values_unsorted, curr_offset, /):
    _preprocess(True, orig_points, shs_half, opacities, cov3Ds, width, height, block_x, block_y, position, rotation,
                focal_x, focal_y, zFar, zNear, points_xy, rgb_depth, conic_opacity, gaussian_keys_unsorted,
                gaussian_values_unsorted, curr_offset)


# ---------------------------------------------------------------------------
# sort (csrc/pybind.cpp:333-349)

def get_sort_buffer_size(num_rendered, /):
    return int(lib().gsr_workspace_size(int(num_rendered)))


def _sort_capacity(num: int, ws_bytes: int, *tensors) -> int:
    cap = min(t.numel() for t in tensors)
    if lib().gsr_workspace_size(cap) <= ws_bytes:
        return cap
    if num <= cap and lib().gsr_workspace_size(num) <= ws_bytes:
        return num
    raise GsrError(_lib.GSR_INVALID_ARG, "sort_gaussian: list_sorting_space is smaller than "
                   "get_sort_buffer_size(%d)" % num)


def sort_gaussian(num_rendered, width, height, block_x, block_y, list_sorting_space, gaussian_keys_unsorted,
                  gaussian_values_unsorted, gaussian_keys_sorted, gaussian_values_sorted, /):
    ws = _dev(list_sorting_space, "list_sorting_space")
    ku = _dev(gaussian_keys_unsorted, "gaussian_keys_unsorted", torch.int64)
    vu = _dev(gaussian_values_unsorted, "gaussian_values_unsorted", torch.int32)
    ks = _dev(gaussian_keys_sorted, "gaussian_keys_sorted", torch.int64)
    vs = _dev(gaussian_values_sorted, "gaussian_values_sorted", torch.int32)
    n = int(num_rendered)
    wsb = ws.numel() * ws.element_size()
    cap = _sort_capacity(n, wsb, ku, vu, ks, vs)
    if n > cap:
        raise GsrError(_lib.GSR_OVERFLOW, "sort_gaussian", n)
    st = lib().gsr_sort(n, None, int(width), int(height), int(block_x), int(block_y), _ptr(ws), wsb, _ptr(ku),
                        _ptr(vu), _ptr(ks), _ptr(vs), cap, _stream(ws.device))
    check(st, "sort_gaussian")


def sort_pairs_bits(num, end_bit, workspace, keys_in, vals_in, keys_out, vals_out):
    """Sort over an explicit bit range [0, end_bit) (library extension)."""
    wsb = workspace.numel() * workspace.element_size()
    cap = _sort_capacity(int(num), wsb, keys_in, vals_in, keys_out, vals_out)
    st = lib().gsr_sort_bits(int(num), None, int(end_bit), _ptr(workspace), wsb, _ptr(keys_in), _ptr(vals_in),
                             _ptr(keys_out), _ptr(vals_out), cap, _stream(workspace.device))
    check(st, "sort_bits")


# ---------------------------------------------------------------------------
# tile ranges / gather

def precompute_tile_ranges(num_rendered, width, height, block_x, block_y, gaussian_keys_sorted, tile_ranges_buf, /):
    ks = _dev(gaussian_keys_sorted, "gaussian_keys_sorted", torch.int64)
    rb = _dev(tile_ranges_buf, "tile_ranges_buf", torch.int32)
    if rb.numel() < 2 * _tiles(width, height, block_x, block_y):
        raise ValueError("tile_ranges_buf holds fewer than 2*tiles ints")
    check(lib().gsr_tile_ranges(int(num_rendered), None, int(width), int(height), int(block_x), int(block_y),
                                _ptr(ks), _ptr(rb), 0, _stream(ks.device)), "precompute_tile_ranges")


def precompute_tile_ranges_scan(num_rendered, width, height, block_x, block_y, gaussian_keys_sorted,
                                tile_ranges_buf, /):
    ks = _dev(gaussian_keys_sorted, "gaussian_keys_sorted", torch.int64)
    rb = _dev(tile_ranges_buf, "tile_ranges_buf", torch.int32)
    if rb.numel() < 2 * _tiles(width, height, block_x, block_y):
        raise ValueError("tile_ranges_buf holds fewer than 2*tiles ints")
    check(lib().gsr_tile_ranges(int(num_rendered), None, int(width), int(height), int(block_x), int(block_y),
                                _ptr(ks), _ptr(rb), 1, _stream(ks.device)), "precompute_tile_ranges_scan")


def gather_features(num_rendered, sorted_values, src_xy, src_rgb_depth, src_conic_opacity, dst_xy, dst_rgb_depth,
                    dst_conic_opacity, /):
    n = int(num_rendered)
    if n <= 0:
        return
    v = _dev(sorted_values, "sorted_values", torch.int32)
    ts = [_dev(t, nm, torch.float32) for t, nm in ((src_xy, "src_xy"), (src_rgb_depth, "src_rgb_depth"),
                                                    (src_conic_opacity, "src_conic_opacity"), (dst_xy, "dst_xy"),
                                                    (dst_rgb_depth, "dst_rgb_depth"),
                                                    (dst_conic_opacity, "dst_conic_opacity"))]
    check(lib().gsr_gather(n, None, _ptr(v), *[_ptr(t) for t in ts], _stream(v.device)), "gather_features")


# ---------------------------------------------------------------------------
# render

def _render(variant, num_rendered, width, height, points_xy, rgb_depth, conic_opacity, keys, values, ranges,
            bg_color, out_color, bx=16, by=16):
    xy = _dev(points_xy, "points_xy", torch.float32)
    rgbd = _dev(rgb_depth, "rgb_depth", torch.float32)
    con = _dev(conic_opacity, "conic_opacity", torch.float32)
    vals = _dev(values, "gaussian_values_sorted", torch.int32)
    out = _dev(out_color, "out_color", torch.uint8)
    if out.numel() < int(width) * int(height) * 3:
        raise ValueError("out_color holds fewer than H*W*3 bytes")
    if keys is not None:
        _dev(keys, "gaussian_keys_sorted", torch.int64)
    if ranges is not None:
        _dev(ranges, "tile_ranges_buf", torch.int32)
    P = min(xy.numel() // 2, rgbd.numel() // 4, con.numel() // 4)
    ws = _render_workspace(out.device)
    st = lib().gsr_render(int(variant), int(num_rendered), None, int(width), int(height), int(bx), int(by), P,
                          _ptr(xy), _ptr(rgbd), _ptr(con), _ptr(keys) if keys is not None else None, _ptr(vals),
                          _ptr(ranges) if ranges is not None else None, _host_floats(bg_color, 3, "bg_color"),
                          _ptr(out), _ptr(ws), _stream(out.device))
    check(st, "render")


R = _lib


def render_16x16(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                 gaussian_values_sorted, bg_color, out_color, /):
    _render(R.RENDER_DEFAULT, num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
            gaussian_keys_sorted, gaussian_values_sorted, None, bg_color, out_color)


def render_16x16_unroll2(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                         gaussian_values_sorted, bg_color, out_color, /):
    _render(R.RENDER_DEFAULT, num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
            gaussian_keys_sorted, gaussian_values_sorted, None, bg_color, out_color)


def render_16x16_split(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                       gaussian_values_sorted, bg_color, out_color, /):
    _render(R.RENDER_SPLIT, num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
            gaussian_keys_sorted, gaussian_values_sorted, None, bg_color, out_color)


def render_24x16_split(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                       gaussian_values_sorted, bg_color, out_color, /):
    _render(R.RENDER_SPLIT, num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
            gaussian_keys_sorted, gaussian_values_sorted, None, bg_color, out_color, 24, 16)


def render_32x16(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                 gaussian_values_sorted, bg_color, out_color, /):
    _render(R.RENDER_DEFAULT, num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
            gaussian_keys_sorted, gaussian_values_sorted, None, bg_color, out_color, 32, 16)


def render_32x16_split(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                       gaussian_values_sorted, bg_color, out_color, /):
    _render(R.RENDER_SPLIT, num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
            gaussian_keys_sorted, gaussian_values_sorted, None, bg_color, out_color, 32, 16)


def render_32x32(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                 gaussian_values_sorted, bg_color, out_color, /):
    _render(R.RENDER_DEFAULT, num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
            gaussian_keys_sorted, gaussian_values_sorted, None, bg_color, out_color, 32, 32)


def render_16x16_preranges(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_values_sorted,
                           tile_ranges_buf, bg_color, out_color, /):
    _render(R.RENDER_RANGES_CADENCE2, num_rendered, width, height, points_xy, rgb_depth, conic_opacity, None,
            gaussian_values_sorted, tile_ranges_buf, bg_color, out_color)


def render_16x16_preranges_smem(num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
                                gaussian_values_sorted, tile_ranges_buf, bg_color, out_color, /):
    _render(R.RENDER_PERSISTENT_RANGES, num_rendered, width, height, points_xy, rgb_depth, conic_opacity, None,
            gaussian_values_sorted, tile_ranges_buf, bg_color, out_color)


def render_16x16_preranges_naive(num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
                                 gaussian_values_sorted, tile_ranges_buf, bg_color, out_color, /):
    _render(R.RENDER_PERSISTENT_RANGES, num_rendered, width, height, points_xy, rgb_depth, conic_opacity, None,
            gaussian_values_sorted, tile_ranges_buf, bg_color, out_color)


def render_16x16_preranges_smem_persistent_lite(num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
                                                gaussian_values_sorted, tile_ranges_buf, bg_color, out_color, /):
    _render(R.RENDER_PERSISTENT_RANGES, num_rendered, width, height, points_xy, rgb_depth, conic_opacity, None,
            gaussian_values_sorted, tile_ranges_buf, bg_color, out_color)


def render_16x16_preranges_smem_persistent_lite_dt(num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
                                                   gaussian_values_sorted, tile_ranges_buf, bg_color, out_color, /):
    _render(R.RENDER_DT, num_rendered, width, height, points_xy, rgb_depth, conic_opacity, None,
            gaussian_values_sorted, tile_ranges_buf, bg_color, out_color)


def render_16x16_preranges_smem_persistent_lite_fused(num_rendered, width, height, points_xy, rgb_depth,
                                                      conic_opacity, gaussian_keys_sorted, gaussian_values_sorted,
                                                      bg_color, out_color, /):
    _render(R.RENDER_PERSISTENT_FUSED, num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
            gaussian_keys_sorted, gaussian_values_sorted, None, bg_color, out_color)


def render_16x16_preranges_smem_v2(num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
                                   gaussian_keys_sorted, gaussian_values_sorted, bg_color, out_color, /):
    # smem_v2 searches its ranges in-kernel and checks every 8 Gaussians
    ranges = torch.empty((_tiles(width, height, 16, 16), 2), dtype=torch.int32, device=points_xy.device)
    precompute_tile_ranges(num_rendered, width, height, 16, 16, gaussian_keys_sorted, ranges)
    _render(R.RENDER_PERSISTENT_RANGES, num_rendered, width, height, points_xy, rgb_depth, conic_opacity, None,
            gaussian_values_sorted, ranges, bg_color, out_color)


def _desc_to_ranges(tile_desc_buf, width, height):
    """int4 tile descriptors {col, row, start, end} -> per-tile [start, end)."""
    T = _tiles(width, height, 16, 16)
    d = _dev(tile_desc_buf, "tile_desc_buf", torch.int32)
    if d.numel() < 4 * T:
        raise GsrError(_lib.GSR_INVALID_ARG, "tile_desc_buf holds fewer than %d descriptors" % T)
    ranges = torch.zeros((T, 2), dtype=torch.int32, device=d.device)
    check(lib().gsr_tile_desc_ranges(_ptr(d), T, (int(width) + 15) // 16, _ptr(ranges), _stream(d.device)),
          "tile descriptors")
    return ranges


def render_16x16_preranges_smem_persistent(num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
                                           gaussian_values_sorted, tile_desc_buf, bg_color, out_color, /):
    _render(R.RENDER_PERSISTENT_RANGES, num_rendered, width, height, points_xy, rgb_depth, conic_opacity, None,
            gaussian_values_sorted, _desc_to_ranges(tile_desc_buf, width, height), bg_color, out_color)


def render_16x16_reordered(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                           gaussian_values_sorted, tile_ranges_buf, tile_order, bg_color, out_color, /):
    _render(R.RENDER_RANGES_CADENCE2, num_rendered, width, height, points_xy, rgb_depth, conic_opacity, None,
            gaussian_values_sorted, tile_ranges_buf, bg_color, out_color)


def render_16x16_reordered_v2(num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
                              gaussian_keys_sorted, gaussian_values_sorted, tile_desc_buf, bg_color, out_color, /):
    _render(R.RENDER_RANGES_CADENCE2, num_rendered, width, height, points_xy, rgb_depth, conic_opacity, None,
            gaussian_values_sorted, _desc_to_ranges(tile_desc_buf, width, height), bg_color, out_color)


def render_16x16_reordered_persistent(num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
                                      gaussian_keys_sorted, gaussian_values_sorted, tile_desc_buf, bg_color,
                                      out_color, /):
    _render(R.RENDER_RANGES_CADENCE2, num_rendered, width, height, points_xy, rgb_depth, conic_opacity, None,
            gaussian_values_sorted, _desc_to_ranges(tile_desc_buf, width, height), bg_color, out_color)


def _topk_render(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                 gaussian_values_sorted, topk_xy, topk_rgb_depth, topk_conic, num_topk, bg_color, out_color):
    """Values with bit 31 set address the top-k feature copies (csrc/ops.h:9-17)."""
    n = int(num_rendered)
    P = points_xy.shape[0]
    k = int(num_topk)
    vals = gaussian_values_sorted[:n]
    flag = vals < 0
    remap = torch.where(flag, (vals & 0x7FFFFFFF) + P, vals).to(torch.int32).contiguous()
    xy = torch.cat([points_xy, topk_xy[:k]]).contiguous()
    rgbd = torch.cat([rgb_depth, topk_rgb_depth[:k]]).contiguous()
    con = torch.cat([conic_opacity, topk_conic[:k]]).contiguous()
    _render(R.RENDER_DEFAULT, n, width, height, xy, rgbd, con, gaussian_keys_sorted, remap, None, bg_color, out_color)


def render_16x16_topk_smem(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                           gaussian_values_sorted, topk_xy, topk_rgb_depth, topk_conic, num_topk, bg_color,
                           out_color, /):
    _topk_render(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                 gaussian_values_sorted, topk_xy, topk_rgb_depth, topk_conic, num_topk, bg_color, out_color)


def render_16x16_topk_smem_persistent(num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
                                      gaussian_keys_sorted, gaussian_values_sorted, topk_xy, topk_rgb_depth,
                                      topk_conic, num_topk, bg_color, out_color, /):
    _topk_render(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                 gaussian_values_sorted, topk_xy, topk_rgb_depth, topk_conic, num_topk, bg_color, out_color)


def render_16x16_topk_smem_persistent_v2(num_rendered, width, height, points_xy, rgb_depth, conic_opacity,
                                         gaussian_keys_sorted, gaussian_values_sorted, topk_xy, topk_rgb_depth,
                                         topk_conic, num_topk, bg_color, out_color, /):
    _topk_render(num_rendered, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                 gaussian_values_sorted, topk_xy, topk_rgb_depth, topk_conic, num_topk, bg_color, out_color)


# ---------------------------------------------------------------------------
# tile-order helpers (ablations; the persistent queue makes them unnecessary)

def get_tile_order_sort_temp_size(total_tiles, /):
    return int(lib().gsr_tile_order_temp_size(int(total_tiles)))


def _tile_order(tile_ranges_buf, total_tiles, x_blocks, morton_bucket, zigzag, tile_desc_buf, tile_order,
                tile_counts_buf, tile_ids_buf, sort_temp, where):
    T = int(total_tiles)
    r = _dev(tile_ranges_buf, "tile_ranges_buf", torch.int32)
    outs = [_dev(tile_order, "tile_order", torch.int32), _dev(tile_counts_buf, "tile_counts_buf", torch.int32),
            _dev(tile_ids_buf, "tile_ids_buf", torch.int32)]
    if r.numel() < 2 * T or any(t.numel() < T for t in outs):
        raise GsrError(_lib.GSR_INVALID_ARG, "%s: a tile buffer holds fewer than %d tiles" % (where, T))
    desc = None
    if tile_desc_buf is not None:
        desc = _dev(tile_desc_buf, "tile_desc_buf", torch.int32)
        if desc.numel() < 4 * T:
            raise GsrError(_lib.GSR_INVALID_ARG, "%s: tile_desc_buf holds fewer than %d descriptors" % (where, T))
    tmp = _dev(sort_temp, "sort_temp")
    st = lib().gsr_tile_order(_ptr(r), T, int(x_blocks), int(morton_bucket), int(zigzag),
                              _ptr(desc) if desc is not None else None, *[_ptr(t) for t in outs], _ptr(tmp),
                              tmp.numel() * tmp.element_size(), _stream(r.device))
    check(st, where)


def compute_tile_order(tile_ranges_buf, total_tiles, tile_order, tile_counts_buf, tile_ids_buf, sort_temp, /):
    """Tiles by descending pair count, ties in index order (render.cu:6959-6979)."""
    _tile_order(tile_ranges_buf, total_tiles, 1, 0, 0, None, tile_order, tile_counts_buf, tile_ids_buf, sort_temp,
                "compute_tile_order")


def compute_tile_order_packed(tile_ranges_buf, total_tiles, x_blocks, tile_desc_buf, tile_order, tile_counts_buf,
                              tile_ids_buf, sort_temp, zigzag_group_size=0, /):
    """The same order plus packed {col, row, start, end} descriptors,
    zig-zagged over groups when zigzag_group_size > 1 (render.cu:6981-7016)."""
    _tile_order(tile_ranges_buf, total_tiles, x_blocks, 0, zigzag_group_size, tile_desc_buf, tile_order,
                tile_counts_buf, tile_ids_buf, sort_temp, "compute_tile_order_packed")


def compute_tile_order_packed_morton(tile_ranges_buf, total_tiles, x_blocks, tile_desc_buf, tile_order,
                                     tile_counts_buf, tile_ids_buf, sort_temp, zigzag_group_size,
                                     morton_bucket_size, /):
    """Order by (count bucket, Morton position) (render.cu:7050-7087)."""
    if int(morton_bucket_size) <= 0:
        raise GsrError(_lib.GSR_INVALID_ARG, "compute_tile_order_packed_morton: morton_bucket_size must be > 0")
    _tile_order(tile_ranges_buf, total_tiles, x_blocks, morton_bucket_size, zigzag_group_size, tile_desc_buf,
                tile_order, tile_counts_buf, tile_ids_buf, sort_temp, "compute_tile_order_packed_morton")


# ---------------------------------------------------------------------------
# ES ("early sorting") two-pass helpers (csrc/pybind.cpp:183-330)

def _es_pass_a(half, orig_points, shs, opacities, cov3Ds, width, height, block_x, block_y, position, rotation,
               focal_x, focal_y, zFar, zNear, points_xy, rgb_depth, conic_opacity, tiles_per_gauss,
               conic_power_raw, depth_natural, rect_bounds):
    pos = _dev(orig_points, "orig_points", torch.float32)
    sh = _dev(shs, "shs", torch.float16 if half else torch.float32)
    op = _dev(opacities, "opacities", torch.float32)
    cov = _dev(cov3Ds, "cov3Ds", torch.float32)
    for t, n in ((points_xy, "points_xy"), (rgb_depth, "rgb_depth"), (conic_opacity, "conic_opacity"),
                 (conic_power_raw, "conic_power_raw"), (depth_natural, "depth_natural")):
        _dev(t, n, torch.float32)
    _dev(tiles_per_gauss, "tiles_per_gauss", torch.int32)
    _dev(rect_bounds, "rect_bounds", torch.int32)
    P = op.numel()
    for t, per, n in ((tiles_per_gauss, 1, "tiles_per_gauss"), (conic_power_raw, 4, "conic_power_raw"),
                      (depth_natural, 1, "depth_natural"), (rect_bounds, 2, "rect_bounds"),
                      (points_xy, 2, "points_xy"), (rgb_depth, 4, "rgb_depth"), (conic_opacity, 4, "conic_opacity")):
        if t.numel() < per * P:
            raise GsrError(_lib.GSR_INVALID_ARG, "preprocess_es_pass_a: %s holds fewer than %d x %d values"
                           % (n, P, per))
    st = lib().gsr_es_pass_a(P, _ptr(pos), _ptr(sh), 1 if half else 0, _ptr(op), _ptr(cov), int(width),
                             int(height), int(block_x), int(block_y), _host_floats(position, 3, "position"),
                             _host_floats(rotation, 9, "rotation"), float(focal_x), float(focal_y), float(zFar),
                             float(zNear), _ptr(points_xy), _ptr(rgb_depth), _ptr(conic_opacity),
                             _ptr(tiles_per_gauss), _ptr(conic_power_raw), _ptr(depth_natural), _ptr(rect_bounds),
                             _stream(op.device))
    check(st, "preprocess_es_pass_a")


def preprocess_es_pass_a(orig_points, shs, opacities, cov3Ds, width, height, block_x, block_y, position, rotation,
                         focal_x, focal_y, zFar, zNear, points_xy, rgb_depth, conic_opacity, tiles_per_gauss,
                         conic_power_raw, depth_natural, rect_bounds, /):
    """ES pass A (csrc/pybind.cpp:183-215): the preprocess without key
    emission; per Gaussian its hit-tile count, raw conic and power, view depth
    (FLT_MAX when culled) and tile rectangle packed as x | y << 16."""
    _es_pass_a(False, orig_points, shs, opacities, cov3Ds, width, height, block_x, block_y, position, rotation,
               focal_x, focal_y, zFar, zNear, points_xy, rgb_depth, conic_opacity, tiles_per_gauss,
               conic_power_raw, depth_natural, rect_bounds)


def preprocess_es_pass_a_half_sh(orig_points, shs_half, opacities, cov3Ds, width, height, block_x, block_y,
                                 position, rotation, focal_x, focal_y, zFar, zNear, points_xy, rgb_depth,
                                 conic_opacity, tiles_per_gauss, conic_power_raw, depth_natural, rect_bounds, /):
    _es_pass_a(True, orig_points, shs_half, opacities, cov3Ds, width, height, block_x, block_y, position, rotation,
               focal_x, focal_y, zFar, zNear, points_xy, rgb_depth, conic_opacity, tiles_per_gauss,
               conic_power_raw, depth_natural, rect_bounds)


def get_es_scan_buffer_size(P, /):
    return int(lib().gsr_es_scan_buffer_size(int(P)))


def es_depth_sort_and_scan(P, tiles_per_gauss, depth_natural, identity_buf, perm_buf, depth_sorted_buf,
                           tiles_per_gauss_sorted_buf, cum_offsets_sorted_buf, total_num_rendered_out,
                           cub_sort_scratch, cub_scan_scratch, /):
    """Stable sort of the Gaussians by view depth, their tile counts in that
    order and its exclusive scan; the total lands in total_num_rendered_out[0]
    on the device (csrc/pybind.cpp:249-292, sort.cu:185-245)."""
    P = int(P)
    ts = [_dev(tiles_per_gauss, "tiles_per_gauss", torch.int32), _dev(depth_natural, "depth_natural", torch.float32),
          _dev(identity_buf, "identity_buf", torch.int32), _dev(perm_buf, "perm_buf", torch.int32),
          _dev(depth_sorted_buf, "depth_sorted_buf", torch.float32),
          _dev(tiles_per_gauss_sorted_buf, "tiles_per_gauss_sorted_buf", torch.int32),
          _dev(cum_offsets_sorted_buf, "cum_offsets_sorted_buf", torch.int32)]
    if any(t.numel() < P for t in ts):
        raise GsrError(_lib.GSR_INVALID_ARG, "es_depth_sort_and_scan: a per-Gaussian buffer holds fewer than %d" % P)
    tot = _dev(total_num_rendered_out, "total_num_rendered_out", torch.int32)
    ws = _dev(cub_sort_scratch, "cub_sort_scratch")
    sc = _dev(cub_scan_scratch, "cub_scan_scratch")
    st = lib().gsr_es_depth_sort_and_scan(P, *[_ptr(t) for t in ts], _ptr(tot), _ptr(ws),
                                          ws.numel() * ws.element_size(), _ptr(sc), sc.numel() * sc.element_size(),
                                          _stream(tot.device))
    check(st, "es_depth_sort_and_scan")


def preprocess_es_pass_b(P, width, height, block_x, block_y, perm, cum_offsets_sorted, tiles_per_gauss_sorted,
                         points_xy, conic_power_raw, rect_bounds, tile_keys_unsorted, gauss_values_unsorted, /):
    """ES pass B (csrc/pybind.cpp:217-247): the (tile id, index) pairs of the
    Gaussians in depth order, each Gaussian's from its scanned offset on.
    Pairs past the output buffers are dropped (the count is known from the
    scan's total)."""
    P = int(P)
    ts = [_dev(perm, "perm", torch.int32), _dev(cum_offsets_sorted, "cum_offsets_sorted", torch.int32),
          _dev(tiles_per_gauss_sorted, "tiles_per_gauss_sorted", torch.int32)]
    xy = _dev(points_xy, "points_xy", torch.float32)
    cpr = _dev(conic_power_raw, "conic_power_raw", torch.float32)
    rb = _dev(rect_bounds, "rect_bounds", torch.int32)
    if any(t.numel() < P for t in ts) or xy.numel() < 2 * P or cpr.numel() < 4 * P or rb.numel() < 2 * P:
        raise GsrError(_lib.GSR_INVALID_ARG, "preprocess_es_pass_b: a per-Gaussian buffer holds fewer than %d" % P)
    tu = _dev(tile_keys_unsorted, "tile_keys_unsorted", torch.int32)
    vu = _dev(gauss_values_unsorted, "gauss_values_unsorted", torch.int32)
    cap = min(tu.numel(), vu.numel())
    st = lib().gsr_es_pass_b(P, int(width), int(height), int(block_x), int(block_y), *[_ptr(t) for t in ts],
                             _ptr(xy), _ptr(cpr), _ptr(rb), _ptr(tu), _ptr(vu), cap, _stream(tu.device))
    check(st, "preprocess_es_pass_b")


def es_tile_sort(num_rendered, width, height, block_x, block_y, tile_keys_unsorted, gauss_values_unsorted,
                 tile_keys_sorted, gauss_values_sorted, gaussian_keys_sorted_out, cub_sort_scratch, /):
    """Stable sort of the pairs by 32-bit tile id over the id's bit width, and
    the 64-bit keys tile << 32 for the range search (csrc/pybind.cpp:294-330,
    sort.cu:247-285)."""
    n = int(num_rendered)
    ts = [_dev(tile_keys_unsorted, "tile_keys_unsorted", torch.int32),
          _dev(gauss_values_unsorted, "gauss_values_unsorted", torch.int32),
          _dev(tile_keys_sorted, "tile_keys_sorted", torch.int32),
          _dev(gauss_values_sorted, "gauss_values_sorted", torch.int32)]
    ko = _dev(gaussian_keys_sorted_out, "gaussian_keys_sorted_out", torch.int64)
    if any(t.numel() < n for t in ts) or ko.numel() < n:
        raise GsrError(_lib.GSR_OVERFLOW, "es_tile_sort", n)
    ws = _dev(cub_sort_scratch, "cub_sort_scratch")
    st = lib().gsr_es_tile_sort(n, int(width), int(height), int(block_x), int(block_y), *[_ptr(t) for t in ts],
                                _ptr(ko), _ptr(ws), ws.numel() * ws.element_size(), _stream(ko.device))
    check(st, "es_tile_sort")


# ---------------------------------------------------------------------------
# fused entry points (csrc/pybind.cpp:876-1149)

_VARIANT_TILES = {"default": None, "unroll2": (16, 16), "split": None}


def _forward(variant, half, orig_points, shs, opacities, cov3Ds, width, height, block_x, block_y, position, rotation,
             focal_x, focal_y, zFar, zNear, curr_offset, list_sorting_space, ku, vu, ks, vs, points_xy, rgb_depth,
             conic_opacity, ranges, bg_color, out_color):
    pos = _dev(orig_points, "orig_points", torch.float32)
    sh = _dev(shs, "shs", torch.float16 if half else torch.float32)
    op = _dev(opacities, "opacities", torch.float32)
    cov = _dev(cov3Ds, "cov3Ds", torch.float32)
    ws = _dev(list_sorting_space, "list_sorting_space")
    for t, nm, dt in ((curr_offset, "curr_offset", torch.int32), (ku, "keys_unsorted", torch.int64),
                      (vu, "values_unsorted", torch.int32), (ks, "keys_sorted", torch.int64),
                      (vs, "values_sorted", torch.int32), (points_xy, "points_xy", torch.float32),
                      (rgb_depth, "rgb_depth", torch.float32), (conic_opacity, "conic_opacity", torch.float32),
                      (out_color, "out_color", torch.uint8)):
        _dev(t, nm, dt)
    if ranges is not None:
        _dev(ranges, "tile_ranges_buf", torch.int32)
    wsb = ws.numel() * ws.element_size()
    cap = _sort_capacity(0, wsb, ku, vu, ks, vs)
    st = lib().gsr_forward(int(variant), op.numel(), _ptr(pos), _ptr(sh), 1 if half else 0, _ptr(op), _ptr(cov),
                           int(width), int(height), int(block_x), int(block_y), _host_floats(position, 3, "position"),
                           _host_floats(rotation, 9, "rotation"), float(focal_x), float(focal_y), float(zFar),
                           float(zNear), _ptr(curr_offset), _ptr(ws), wsb, _ptr(ku), _ptr(vu), _ptr(ks), _ptr(vs), cap,
                           _ptr(points_xy), _ptr(rgb_depth), _ptr(conic_opacity),
                           _ptr(ranges) if ranges is not None else None, _host_floats(bg_color, 3, "bg_color"),
                           _ptr(out_color), _stream(ws.device))
    check(st, "forward")
    return _read_status(ws, curr_offset, cap, "forward")


def depth_first_scratch_size(P):
    """Bytes of per-Gaussian scratch the depth-first forward needs (library extension)."""
    return int(lib().gsr_depth_first_scratch_size(int(P)))


def forward_depth_first(variant, half, orig_points, shs, opacities, cov3Ds, width, height, block_x, block_y, position,
                        rotation, focal_x, focal_y, zFar, zNear, curr_offset, list_sorting_space, scene_scratch,
                        tiles_unsorted, values_unsorted, tiles_sorted, values_sorted, points_xy, rgb_depth,
                        conic_opacity, ranges, bg_color, out_color):
    """Depth-first ("early sorting") forward in one call (library extension;
    the reference's two-pass ES pipeline, csrc/cuda_rasterizer/preprocess.cu:673-1248,
    sort.cu:151-285).  Tile ids and values are int32 tensors of the key
    capacity; returns the pair count M."""
    pos = _dev(orig_points, "orig_points", torch.float32)
    sh = _dev(shs, "shs", torch.float16 if half else torch.float32)
    op = _dev(opacities, "opacities", torch.float32)
    cov = _dev(cov3Ds, "cov3Ds", torch.float32)
    ws = _dev(list_sorting_space, "list_sorting_space")
    sc = _dev(scene_scratch, "scene_scratch")
    for t, nm, dt in ((curr_offset, "curr_offset", torch.int32), (tiles_unsorted, "tiles_unsorted", torch.int32),
                      (values_unsorted, "values_unsorted", torch.int32), (tiles_sorted, "tiles_sorted", torch.int32),
                      (values_sorted, "values_sorted", torch.int32), (points_xy, "points_xy", torch.float32),
                      (rgb_depth, "rgb_depth", torch.float32), (conic_opacity, "conic_opacity", torch.float32),
                      (out_color, "out_color", torch.uint8)):
        _dev(t, nm, dt)
    if ranges is not None:
        _dev(ranges, "tile_ranges_buf", torch.int32)
    wsb = ws.numel() * ws.element_size()
    cap = _sort_capacity(0, wsb, tiles_unsorted, values_unsorted, tiles_sorted, values_sorted)
    st = lib().gsr_forward_depth_first(
        int(variant), op.numel(), _ptr(pos), _ptr(sh), 1 if half else 0, _ptr(op), _ptr(cov), int(width),
        int(height), int(block_x), int(block_y), _host_floats(position, 3, "position"),
        _host_floats(rotation, 9, "rotation"), float(focal_x), float(focal_y), float(zFar), float(zNear),
        _ptr(curr_offset), _ptr(ws), wsb, _ptr(sc), sc.numel() * sc.element_size(), _ptr(tiles_unsorted),
        _ptr(values_unsorted), _ptr(tiles_sorted), _ptr(values_sorted), cap, _ptr(points_xy), _ptr(rgb_depth),
        _ptr(conic_opacity), _ptr(ranges) if ranges is not None else None, _host_floats(bg_color, 3, "bg_color"),
        _ptr(out_color), _stream(ws.device))
    check(st, "forward_depth_first")
    return _read_status(ws, curr_offset, cap, "forward_depth_first")


def _variant_code(render_variant: str, block_x: int, block_y: int) -> int:
    if render_variant in ("default", "unroll2", "split"):
        return R.RENDER_DEFAULT
    raise ValueError("unsupported render_variant %r for the fused forward" % render_variant)


def forward_fused(orig_points, shs, opacities, cov3Ds, width, height, block_x, block_y, position, rotation, focal_x,
                  focal_y, zFar, zNear, render_variant, curr_offset, list_sorting_space, gaussian_keys_unsorted,
                  gaussian_values_unsorted, gaussian_keys_sorted, gaussian_values_sorted, points_xy, rgb_depth,
                  conic_opacity, bg_color, out_color, /):
    v = _variant_code(render_variant, block_x, block_y)
    return _forward(v, False, orig_points, shs, opacities, cov3Ds, width, height, block_x, block_y, position,
                    rotation, focal_x, focal_y, zFar, zNear, curr_offset, list_sorting_space, gaussian_keys_unsorted,
                    gaussian_values_unsorted, gaussian_keys_sorted, gaussian_values_sorted, points_xy, rgb_depth,
                    conic_opacity, None, bg_color, out_color)


def forward_fused_e2e(orig_points, shs_half, opacities, cov3Ds, width, height, block_x, block_y, position, rotation,
                      focal_x, focal_y, zFar, zNear, curr_offset, list_sorting_space, gaussian_keys_unsorted,
                      gaussian_values_unsorted, gaussian_keys_sorted, gaussian_values_sorted, points_xy, rgb_depth,
                      conic_opacity, bg_color, out_color, /):
    return _forward(R.RENDER_PERSISTENT_FUSED, True, orig_points, shs_half, opacities, cov3Ds, width, height, block_x,
                    block_y, position, rotation, focal_x, focal_y, zFar, zNear, curr_offset, list_sorting_space,
                    gaussian_keys_unsorted, gaussian_values_unsorted, gaussian_keys_sorted, gaussian_values_sorted,
                    points_xy, rgb_depth, conic_opacity, None, bg_color, out_color)


def forward_fused_e2e_preranges(orig_points, shs_half, opacities, cov3Ds, width, height, block_x, block_y, position,
                                rotation, focal_x, focal_y, zFar, zNear, curr_offset, list_sorting_space,
                                gaussian_keys_unsorted, gaussian_values_unsorted, gaussian_keys_sorted,
                                gaussian_values_sorted, points_xy, rgb_depth, conic_opacity, tile_ranges_buf,
                                bg_color, out_color, /):
    return _forward(R.RENDER_PERSISTENT_RANGES, True, orig_points, shs_half, opacities, cov3Ds, width, height,
                    block_x, block_y, position, rotation, focal_x, focal_y, zFar, zNear, curr_offset,
                    list_sorting_space, gaussian_keys_unsorted, gaussian_values_unsorted, gaussian_keys_sorted,
                    gaussian_values_sorted, points_xy, rgb_depth, conic_opacity, tile_ranges_buf, bg_color, out_color)


def sort_and_render(width, height, block_x, block_y, render_variant, curr_offset, list_sorting_space,
                    gaussian_keys_unsorted, gaussian_values_unsorted, gaussian_keys_sorted, gaussian_values_sorted,
                    points_xy, rgb_depth, conic_opacity, bg_color, out_color, /):
    ws = _dev(list_sorting_space, "list_sorting_space")
    n = _read_status(ws, _dev(curr_offset, "curr_offset", torch.int32),
                     min(gaussian_keys_unsorted.numel(), gaussian_keys_sorted.numel()), "sort_and_render")
    sort_gaussian(n, width, height, block_x, block_y, list_sorting_space, gaussian_keys_unsorted,
                  gaussian_values_unsorted, gaussian_keys_sorted, gaussian_values_sorted)
    if render_variant in ("default", "unroll2", "split"):
        _render(R.RENDER_DEFAULT, n, width, height, points_xy, rgb_depth, conic_opacity, gaussian_keys_sorted,
                gaussian_values_sorted, None, bg_color, out_color, block_x, block_y)
    return n
