"""ctypes front end of the FP64 CPU oracle (``gsr_oracle.c``) -- TEST INFRASTRUCTURE.

Only the test suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline leg use this module, and only as the checker; the product path
(``polysplat_gb300``) never imports it.

The C source restates the reference's equations in double precision; each
function there cites the reference file:line it follows.  ``build()``
compiles it with the host ``gcc`` into ``oracle/_build/``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libgsr_oracle.so")
SRC = os.path.join(HERE, "gsr_oracle.c")

_lib = None


def build(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-o", tmp, SRC, "-lpthread", "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        i32, i64, f32 = ctypes.c_int, ctypes.c_int64, ctypes.c_float
        L.ora_scene_transform.argtypes = [i32, P, P, P, P, P]
        L.ora_scene_transform.restype = None
        L.ora_preprocess.argtypes = [i32, P, P, P, P, i32, i32, i32, i32, P, P, f32, f32, f32, f32,
                                     P, P, P, P, P, P, i64, i32]
        L.ora_preprocess.restype = i64
        L.ora_higher_msb.argtypes = [ctypes.c_uint32]
        L.ora_higher_msb.restype = ctypes.c_uint32
        L.ora_sort_pairs.argtypes = [i64, P, P, P, P, i32]
        L.ora_sort_pairs.restype = None
        L.ora_tile_ranges_bsearch.argtypes = [i64, P, i32, P]
        L.ora_tile_ranges_bsearch.restype = None
        L.ora_tile_ranges_scan.argtypes = [i64, P, i32, P]
        L.ora_tile_ranges_scan.restype = None
        L.ora_gather.argtypes = [i64, P, P, P, P, P, P, P]
        L.ora_gather.restype = None
        L.ora_render.argtypes = [i64, P, P, P, P, P, i32, i32, i32, i32, i32, i32, P, P, P, i32]
        L.ora_render.restype = None
        L.ora_image_fp64.argtypes = [i32, P, P, P, P, P, i32, i32, P, P, ctypes.c_double, ctypes.c_double, P, i32, P,
                                     P, i32]
        L.ora_image_fp64.restype = ctypes.c_double
        L.ora_image_fp64_masked.argtypes = [i32, P, P, P, P, P, i32, i32, P, P, ctypes.c_double, ctypes.c_double, P,
                                            i32, P, P, P, P, i32]
        L.ora_image_fp64_masked.restype = ctypes.c_double
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be contiguous"
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def nthreads_default() -> int:
    return max(1, os.cpu_count() or 1)


def scene_transform(log_scales, quats, logits):
    """Raw parameters -> (opacity [P], cov3d [P,6]) (``csrc/pybind.cpp:22-56,105-117``)."""
    ls, q, lg = _c(log_scales, np.float32), _c(quats, np.float32), _c(logits, np.float32)
    n = lg.shape[0]
    op = np.empty(n, np.float32)
    cov = np.empty((n, 6), np.float32)
    lib().ora_scene_transform(n, _p(ls), _p(q), _p(lg), _p(op), _p(cov))
    return op, cov


def camera_args(cam):
    return (_c(cam.position, np.float32).reshape(3), _c(cam.rotation, np.float32).reshape(9))


def preprocess(pos, shs, opacity, cov3d, W, H, cam_pos, cam_rot, fx, fy, bx=16, by=16,
               zfar=100.0, znear=0.01, capacity=None, nthreads=None):
    """Returns dict(num, keys, vals, xy, rgbd, con, emitted)."""
    pos, shs = _c(pos, np.float32), _c(shs, np.float32).reshape(-1, 48)
    op, cov = _c(opacity, np.float32), _c(cov3d, np.float32)
    P = op.shape[0]
    cp, cr = _c(cam_pos, np.float32).reshape(3), _c(cam_rot, np.float32).reshape(9)
    xy = np.zeros((P, 2), np.float32)
    rgbd = np.zeros((P, 4), np.float32)
    con = np.zeros((P, 4), np.float32)
    emitted = np.zeros(P, np.uint8)
    nt = nthreads or nthreads_default()
    if capacity is None:
        m = lib().ora_preprocess(P, _p(pos), _p(shs), _p(op), _p(cov), W, H, bx, by, _p(cp), _p(cr),
                                 fx, fy, zfar, znear, _p(xy), _p(rgbd), _p(con), _p(emitted),
                                 None, None, 0, nt)
        capacity = m
    keys = np.zeros(max(capacity, 1), np.uint64)
    vals = np.zeros(max(capacity, 1), np.uint32)
    m = lib().ora_preprocess(P, _p(pos), _p(shs), _p(op), _p(cov), W, H, bx, by, _p(cp), _p(cr),
                             fx, fy, zfar, znear, _p(xy), _p(rgbd), _p(con), _p(emitted),
                             _p(keys), _p(vals), capacity, nt)
    k = min(m, capacity)
    return dict(num=int(m), keys=keys[:k], vals=vals[:k], xy=xy, rgbd=rgbd, con=con,
                emitted=emitted.astype(bool))


def higher_msb(n: int) -> int:
    return int(lib().ora_higher_msb(n))


def end_bit_for(W, H, bx=16, by=16) -> int:
    gx, gy = (W + bx - 1) // bx, (H + by - 1) // by
    return 32 + higher_msb(gx * gy)


def sort_pairs(keys, vals, end_bit=64):
    k, v = _c(keys, np.uint64), _c(vals, np.uint32)
    n = k.shape[0]
    ko = np.empty_like(k)
    vo = np.empty_like(v)
    lib().ora_sort_pairs(n, _p(k), _p(v), _p(ko), _p(vo), end_bit)
    return ko, vo


def tile_ranges(keys, tiles, scan=False):
    k = _c(keys, np.uint64)
    r = np.empty((tiles, 2), np.int32)
    fn = lib().ora_tile_ranges_scan if scan else lib().ora_tile_ranges_bsearch
    fn(k.shape[0], _p(k), tiles, _p(r))
    return r


def gather(vals, xy, rgbd, con):
    v = _c(vals, np.uint32)
    xy, rgbd, con = _c(xy, np.float32), _c(rgbd, np.float32), _c(con, np.float32)
    n = v.shape[0]
    dxy = np.empty((n, 2), np.float32)
    drgbd = np.empty((n, 4), np.float32)
    dcon = np.empty((n, 4), np.float32)
    lib().ora_gather(n, _p(v), _p(xy), _p(rgbd), _p(con), _p(dxy), _p(drgbd), _p(dcon))
    return dxy, drgbd, dcon


def render(vals, ranges, xy, rgbd, con, W, H, bg=(0.0, 0.0, 0.0), bx=16, by=16, cadence=8,
           dt=False, nthreads=None, want_counts=False):
    v, r = _c(vals, np.uint32), _c(ranges, np.int32)
    xy, rgbd, con = _c(xy, np.float32), _c(rgbd, np.float32), _c(con, np.float32)
    bgc = _c(bg, np.float32).reshape(3)
    out = np.zeros((H, W, 3), np.uint8)
    tiles = ((W + bx - 1) // bx) * ((H + by - 1) // by)
    counts = np.zeros(tiles, np.int64) if want_counts else None
    lib().ora_render(v.shape[0], _p(v), _p(r), _p(xy), _p(rgbd), _p(con), W, H, bx, by, cadence,
                     1 if dt else 0, _p(bgc), _p(out), _p(counts) if counts is not None else None,
                     nthreads or nthreads_default())
    return (out, counts) if want_counts else out


def forward(pos, shs, opacity, cov3d, cam, bg=(0.0, 0.0, 0.0), bx=16, by=16, cadence=8,
            half_sh=False, nthreads=None):
    """Whole forward: preprocess -> sort -> ranges -> blend.  Returns (image, dict)."""
    shs = _c(shs, np.float32).reshape(-1, 48)
    if half_sh:
        shs = shs.astype(np.float16).astype(np.float32)
    cp, cr = camera_args(cam)
    pre = preprocess(pos, shs, opacity, cov3d, cam.width, cam.height, cp, cr, cam.fx, cam.fy,
                     bx, by, nthreads=nthreads)
    eb = end_bit_for(cam.width, cam.height, bx, by)
    ks, vs = sort_pairs(pre["keys"], pre["vals"], eb)
    tiles = ((cam.width + bx - 1) // bx) * ((cam.height + by - 1) // by)
    rng = tile_ranges(ks, tiles)
    img = render(vs, rng, pre["xy"], pre["rgbd"], pre["con"], cam.width, cam.height, bg, bx, by,
                 cadence, nthreads=nthreads)
    pre.update(keys_sorted=ks, vals_sorted=vs, ranges=rng, end_bit=eb)
    return img, pre


def image_fp64(means, log_scales, quats, logits, shs, cam, bg=(0.0, 0.0, 0.0), cadence=8, target=None,
               nthreads=None):
    """The float image of one camera in double end to end from raw parameters
    (gsr_oracle.c ora_image_fp64) and, with `target`, its L2 loss.
    Returns (loss, image [H,W,3] float64)."""
    f8 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    m, ls, q, lg, sh = f8(means), f8(log_scales), f8(quats), f8(logits), f8(shs).reshape(-1, 48)
    P = lg.shape[0]
    img = np.zeros((cam.height, cam.width, 3), np.float64)
    cp, cr = _c(cam.position, np.float32).reshape(3), _c(cam.rotation, np.float32).reshape(9)
    b = f8(bg).reshape(3)
    tgt = f8(target) if target is not None else None
    loss = lib().ora_image_fp64(P, _p(m), _p(ls), _p(q), _p(lg), _p(sh), cam.width, cam.height, _p(cp), _p(cr),
                                float(cam.fx), float(cam.fy), _p(b), int(cadence),
                                _p(tgt) if tgt is not None else None, _p(img), nthreads or nthreads_default())
    return float(loss), img



def _spread16(v):
    v = v.astype(np.uint32) & np.uint32(0xFFFF)
    for shift, mask in ((8, 0x00FF00FF), (4, 0x0F0F0F0F), (2, 0x33333333), (1, 0x55555555)):
        v = (v | (v << np.uint32(shift))) & np.uint32(mask)
    return v


def tile_order(ranges, x_blocks, morton_bucket=0, zigzag=0):
    """Tile reordering of the reference's reordered renders, in numpy.

    Sort key per tile t: its pair count ranges[t,1] - ranges[t,0]
    (extractTileCounts, render.cu:4414-4426), or with morton_bucket > 0
    (min(count // bucket, 0xFFFF) << 16) | (0xFFFF - Morton(x, y) & 0xFFFF)
    (extractTileCountsMorton, render.cu:4496-4520).  Stable descending sort
    of (key, tile id) (cub SortPairsDescending, render.cu:6973-6977).
    Descriptors {col, row, start, end} in that order (gatherTileDesc,
    render.cu:4813-4831); with zigzag > 1 odd groups of `zigzag` positions
    read their slice backwards (gatherTileDescZigzag, render.cu:4838-4866).

    Returns (order, sorted_keys, ids, desc) as uint32/int32 arrays."""
    r = np.asarray(ranges, dtype=np.int64).reshape(-1, 2)
    T = r.shape[0]
    key = ((r[:, 1] - r[:, 0]) & 0xFFFFFFFF).astype(np.uint32)
    t = np.arange(T, dtype=np.int64)
    if morton_bucket > 0:
        bucket = np.minimum(key // np.uint32(morton_bucket), np.uint32(0xFFFF)).astype(np.uint32)
        morton = (_spread16(t % x_blocks) | (_spread16(t // x_blocks) << np.uint32(1))) & np.uint32(0xFFFF)
        key = (bucket << np.uint32(16)) | (np.uint32(0xFFFF) - morton)
    order = np.argsort(-key.astype(np.int64), kind="stable").astype(np.uint32)
    src = t.copy()
    if zigzag > 1:
        g = t // zigzag
        base = g * zigzag
        length = np.minimum(base + zigzag, T) - base
        src = np.where(g % 2 == 1, base + (length - 1 - (t - base)), t)
        src = np.minimum(src, T - 1)
    ids = order[src].astype(np.int64)
    desc = np.stack([ids % x_blocks, ids // x_blocks, r[ids, 0], r[ids, 1]], axis=1).astype(np.int32)
    return order, key[order], t.astype(np.uint32), desc


def image_fp64_masked(means, log_scales, quats, logits, shs, cam, tile_mask=None, bg=(0.0, 0.0, 0.0), cadence=8,
                      target=None, nthreads=None):
    """image_fp64 restricted to the 16x16 tiles where `tile_mask` (uint8
    [tiles], row-major; None = every tile) is set: the loss sums over those
    tiles' pixels only.  Returns (loss, image [H,W,3], rects [P,4]) with each
    Gaussian's tile rectangle x0, y0, x1, y1 (zeros when culled)."""
    f8 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    m, ls, q, lg, sh = f8(means), f8(log_scales), f8(quats), f8(logits), f8(shs).reshape(-1, 48)
    P = lg.shape[0]
    img = np.zeros((cam.height, cam.width, 3), np.float64)
    rects = np.zeros((P, 4), np.int32)
    cp, cr = _c(cam.position, np.float32).reshape(3), _c(cam.rotation, np.float32).reshape(9)
    b = f8(bg).reshape(3)
    tgt = f8(target) if target is not None else None
    mask = np.ascontiguousarray(tile_mask, dtype=np.uint8) if tile_mask is not None else None
    loss = lib().ora_image_fp64_masked(P, _p(m), _p(ls), _p(q), _p(lg), _p(sh), cam.width, cam.height, _p(cp),
                                       _p(cr), float(cam.fx), float(cam.fy), _p(b), int(cadence),
                                       _p(tgt) if tgt is not None else None, _p(mask) if mask is not None else None,
                                       _p(rects), _p(img), nthreads or nthreads_default())
    return float(loss), img, rects

