"""Python front end of the reference-kernel runner -- TEST INFRASTRUCTURE.

Runs the reference rasterizer's own CUDA kernels (compiled from its sources by
``ref_build.py``) on torch tensors, with the same camera matrices the library
computes, so tests can compare both implementations on identical inputs.
"""
from __future__ import annotations

import ctypes
import os

import torch

from . import ref_build

_lib = None


def available() -> bool:
    return all(os.path.exists(os.path.join(ref_build.OUT, f)) for f in ("preprocess.cubin", "render.cubin"))


def lib():
    global _lib
    if _lib is None:
        path = ref_build.build_runner()
        L = ctypes.CDLL(path)
        P, i32, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.ref_open.argtypes = [ctypes.c_char_p]
        L.ref_preprocess.argtypes = [i32, P, P, P, i32, P, P, P, i32, i32, i32, i32, f32, f32, f32, f32,
                                     P, P, P, P, P, P, P, P]
        L.ref_tile_ranges.argtypes = [i32, P, i32, P, P]
        L.ref_render.argtypes = [i32, i32, i32, i32, P, P, P, P, P, P, P, P, P]
        L.ref_has_tile_counter.restype = i32
        L.ref_sort_temp_bytes.argtypes = [i32]
        L.ref_sort_temp_bytes.restype = ctypes.c_size_t
        L.ref_sort.argtypes = [i32, i32, P, ctypes.c_size_t, P, P, P, P, P]
        L.ref_forward_e2e.argtypes = [i32, P, P, P, P, P, P, P, i32, i32, f32, f32, P, P, ctypes.c_size_t,
                                      P, P, P, P, P, P, P, P, P, P]
        sz = ctypes.c_size_t
        L.ref_es_pass_a.argtypes = [i32, P, P, P, i32, P, P, P, i32, i32, i32, i32, f32, f32, f32, f32,
                                    P, P, P, P, P, P, P, P, P]
        L.ref_es_pass_b.argtypes = [i32, i32, i32, i32, i32, P, P, P, P, P, P, P, P, P]
        for n in ("ref_es_depth_sort_temp_bytes", "ref_es_scan_temp_bytes", "ref_es_tile_sort_temp_bytes"):
            getattr(L, n).argtypes = [i32]
            getattr(L, n).restype = sz
        L.ref_es_depth_sort_and_scan.argtypes = [i32, P, P, P, P, P, P, P, P, P, sz, P, sz, P]
        L.ref_es_tile_sort.argtypes = [i32, i32, i32, i32, i32, P, P, P, P, P, P, sz, P]
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        rc = L.ref_open(ref_build.OUT.encode())
        if rc != 0:
            raise RuntimeError("reference kernels could not be loaded (code %d)" % rc)
        _lib = L
    return _lib


def _f(vals, n):
    return (ctypes.c_float * n)(*[float(v) for v in vals])


def camera_matrices(W, H, pos, rot, fx, fy, zfar=100.0, znear=0.01):
    """View/projection matrices (column-major) for the reference's kernels.

    The reference's own host functions (getViewMatrix / getProjectionMatrix,
    preprocess.cu:643-671) are not available where the GPU runs; the
    library's gsr_camera_matrices stands in for them, and
    tests/test_ref_host.py pins it bit for bit to the reference's functions
    on 256 cameras (tests/golden/host_reference.npz)."""
    from polysplat_gb300._lib import lib as gsr_lib

    view = (ctypes.c_float * 16)()
    proj = (ctypes.c_float * 16)()
    gsr_lib().gsr_camera_matrices(int(W), int(H), _f(pos, 3), _f(list(map(float, __import__("numpy").asarray(
        rot, dtype="float32").reshape(9))), 9), float(fx), float(fy), float(zfar), float(znear), view, proj)
    return list(view), list(proj)


def _tan_fov(size, f):
    """size / (2 f) in float32, as the host launcher computes it (preprocess.cu:1265-1266)."""
    import numpy as np

    return float(np.float32(size) / (np.float32(2.0) * np.float32(f)))


def preprocess(scene, cam, half, xy, cov3d, rgbd, con, counter, keys, vals, bx=16, by=16):
    view, proj = camera_matrices(cam.width, cam.height, cam.position, cam.rotation, cam.fx, cam.fy)
    sh = scene.shs_half if half else scene.shs
    rc = lib().ref_preprocess(scene.num_vertex, scene.position.data_ptr(), scene.opacity.data_ptr(), sh.data_ptr(),
                              1 if half else 0, _f(view, 16), _f(proj, 16), _f(cam.position, 3), cam.width,
                              cam.height, bx, by, _tan_fov(cam.width, cam.fx), _tan_fov(cam.height, cam.fy), cam.fx,
                              cam.fy, xy.data_ptr(), cov3d.data_ptr(), rgbd.data_ptr(), con.data_ptr(),
                              counter.data_ptr(), keys.data_ptr(), vals.data_ptr(),
                              torch.cuda.current_stream().cuda_stream)
    if rc:
        raise RuntimeError("reference preprocess launch failed (%d)" % rc)


def tile_ranges(M, keys, tiles, ranges):
    rc = lib().ref_tile_ranges(int(M), keys.data_ptr(), int(tiles), ranges.data_ptr(),
                               torch.cuda.current_stream().cuda_stream)
    if rc:
        raise RuntimeError("reference tile ranges failed (%d)" % rc)


def sort_temp_bytes(n):
    return int(lib().ref_sort_temp_bytes(int(n)))


def sort(n, end_bit, temp, ku, vu, ks, vs):
    """The reference's sort call (CUB SortPairs over bits [0, end_bit))."""
    rc = lib().ref_sort(int(n), int(end_bit), temp.data_ptr(), temp.numel(), ku.data_ptr(), vu.data_ptr(),
                        ks.data_ptr(), vs.data_ptr(), torch.cuda.current_stream().cuda_stream)
    if rc:
        raise RuntimeError("reference sort failed (%d)" % rc)


class Pipeline:
    """The reference's E2E forward (pybind.cpp:1085-1149) on preallocated buffers."""

    def __init__(self, scene, cam, capacity):
        dev = scene.position.device
        P = scene.num_vertex
        self.scene, self.cam, self.cap = scene, cam, capacity
        self.view, self.proj = camera_matrices(cam.width, cam.height, cam.position, cam.rotation, cam.fx, cam.fy)
        self.view_c, self.proj_c = _f(self.view, 16), _f(self.proj, 16)
        self.cam_c = _f(cam.position, 3)
        self.counter = torch.zeros(1, dtype=torch.int32, device=dev)
        self.temp = torch.zeros(sort_temp_bytes(capacity), dtype=torch.int8, device=dev)
        self.ku = torch.zeros(capacity, dtype=torch.int64, device=dev)
        self.vu = torch.zeros(capacity, dtype=torch.int32, device=dev)
        self.ks = torch.zeros(capacity, dtype=torch.int64, device=dev)
        self.vs = torch.zeros(capacity, dtype=torch.int32, device=dev)
        self.xy = torch.zeros((P, 2), device=dev)
        self.rgbd = torch.zeros((P, 4), device=dev)
        self.con = torch.zeros((P, 4), device=dev)
        self.out = torch.zeros((cam.height, cam.width, 3), dtype=torch.uint8, device=dev)
        self.bg = _f([0.0, 0.0, 0.0], 3)

    def set_view(self, scene, cam):
        """Point the pipeline at another scene and camera (key buffers kept;
        feature buffers grown when the scene is larger)."""
        dev = scene.position.device
        P = scene.num_vertex
        if P > self.xy.shape[0]:
            self.xy = torch.zeros((P, 2), device=dev)
            self.rgbd = torch.zeros((P, 4), device=dev)
            self.con = torch.zeros((P, 4), device=dev)
        self.scene, self.cam = scene, cam
        self.view, self.proj = camera_matrices(cam.width, cam.height, cam.position, cam.rotation, cam.fx, cam.fy)
        self.view_c, self.proj_c = _f(self.view, 16), _f(self.proj, 16)
        self.cam_c = _f(cam.position, 3)
        self.out = torch.zeros((cam.height, cam.width, 3), dtype=torch.uint8, device=dev)

    def forward(self):
        s, c = self.scene, self.cam
        n = lib().ref_forward_e2e(s.num_vertex, s.position.data_ptr(), s.shs_half.data_ptr(), s.opacity.data_ptr(),
                                  s.cov3d.data_ptr(), self.view_c, self.proj_c, self.cam_c, c.width, c.height,
                                  c.fx, c.fy, self.counter.data_ptr(), self.temp.data_ptr(), self.temp.numel(),
                                  self.ku.data_ptr(), self.vu.data_ptr(), self.ks.data_ptr(), self.vs.data_ptr(),
                                  self.xy.data_ptr(), self.rgbd.data_ptr(), self.con.data_ptr(), self.bg,
                                  self.out.data_ptr(), torch.cuda.current_stream().cuda_stream)
        if n < 0:
            raise RuntimeError("reference forward failed (%d)" % -n)
        if n > self.cap:
            raise RuntimeError("reference forward overflowed its key buffers (%d keys)" % n)
        return n


def render(which, M, W, H, xy, rgbd, con, keys, vals, ranges, bg, out):
    """which: 'lite' (ranges), 'fused' (keys), 'default', '32x16', '32x32',
    'unroll2', 'split16', 'split24', 'split32' (keys)."""
    code = {"lite": 0, "fused": 1, "default": 2, "32x16": 3, "32x32": 4, "unroll2": 5, "split16": 6,
            "split24": 7, "split32": 8}[which]
    rc = lib().ref_render(code, int(M), int(W), int(H), xy.data_ptr(), rgbd.data_ptr(), con.data_ptr(),
                          keys.data_ptr() if keys is not None else None, vals.data_ptr(),
                          ranges.data_ptr() if ranges is not None else None, _f(bg, 3), out.data_ptr(),
                          torch.cuda.current_stream().cuda_stream)
    if rc:
        raise RuntimeError("reference render failed (%d)" % rc)


def es_chain(scene, cam, half, cap, bx=16, by=16):
    """The reference's ES steps in its order (example.py:495-580): its pass A
    kernel, the CUB depth sort and scan of es_depth_sort_and_scan, its pass B
    kernel and the CUB tile sort of es_tile_sort.  Returns the buffers."""
    dev = scene.position.device
    P = scene.num_vertex
    i32, f32 = torch.int32, torch.float32
    z = lambda *shape, dtype=f32: torch.zeros(shape, device=dev, dtype=dtype)
    b = dict(xy=z(P, 2), rgbd=z(P, 4), con=z(P, 4), tiles_per_gauss=z(P, dtype=i32), conic_power_raw=z(P, 4),
             depth_natural=z(P), rect_bounds=z(P, 2, dtype=i32), identity=z(P, dtype=i32), perm=z(P, dtype=i32),
             depth_sorted=z(P), tiles_sorted=z(P, dtype=i32), cum=z(P, dtype=i32), total=z(1, dtype=i32),
             tku=z(cap, dtype=i32), vu=z(cap, dtype=i32), tks=z(cap, dtype=i32), vs=z(cap, dtype=i32),
             ks=z(cap, dtype=torch.int64))
    L = lib()
    st = torch.cuda.current_stream().cuda_stream
    view, proj = camera_matrices(cam.width, cam.height, cam.position, cam.rotation, cam.fx, cam.fy)
    sh = scene.shs_half if half else scene.shs
    rc = L.ref_es_pass_a(P, scene.position.data_ptr(), scene.opacity.data_ptr(), sh.data_ptr(), 1 if half else 0,
                         _f(view, 16), _f(proj, 16), _f(cam.position, 3), cam.width, cam.height, bx, by,
                         _tan_fov(cam.width, cam.fx), _tan_fov(cam.height, cam.fy), cam.fx, cam.fy,
                         b["xy"].data_ptr(), scene.cov3d.data_ptr(), b["rgbd"].data_ptr(), b["con"].data_ptr(),
                         b["tiles_per_gauss"].data_ptr(), b["conic_power_raw"].data_ptr(),
                         b["depth_natural"].data_ptr(), b["rect_bounds"].data_ptr(), st)
    if rc:
        raise RuntimeError("reference ES pass A failed (%d)" % rc)
    t_sort = torch.zeros(int(L.ref_es_depth_sort_temp_bytes(P)), dtype=torch.int8, device=dev)
    t_scan = torch.zeros(int(L.ref_es_scan_temp_bytes(P)), dtype=torch.int8, device=dev)
    rc = L.ref_es_depth_sort_and_scan(P, b["tiles_per_gauss"].data_ptr(), b["depth_natural"].data_ptr(),
                                      b["identity"].data_ptr(), b["perm"].data_ptr(), b["depth_sorted"].data_ptr(),
                                      b["tiles_sorted"].data_ptr(), b["cum"].data_ptr(), b["total"].data_ptr(),
                                      t_sort.data_ptr(), t_sort.numel(), t_scan.data_ptr(), t_scan.numel(), st)
    if rc:
        raise RuntimeError("reference ES depth sort / scan failed (%d)" % rc)
    m = int(b["total"].cpu()[0])
    if m > cap:
        raise RuntimeError("reference ES pairs (%d) exceed the buffers (%d)" % (m, cap))
    rc = L.ref_es_pass_b(P, cam.width, cam.height, bx, by, b["perm"].data_ptr(), b["cum"].data_ptr(),
                         b["tiles_sorted"].data_ptr(), b["xy"].data_ptr(), b["conic_power_raw"].data_ptr(),
                         b["rect_bounds"].data_ptr(), b["tku"].data_ptr(), b["vu"].data_ptr(), st)
    if rc:
        raise RuntimeError("reference ES pass B failed (%d)" % rc)
    t_tile = torch.zeros(int(L.ref_es_tile_sort_temp_bytes(max(1, m))), dtype=torch.int8, device=dev)
    rc = L.ref_es_tile_sort(m, cam.width, cam.height, bx, by, b["tku"].data_ptr(), b["vu"].data_ptr(),
                            b["tks"].data_ptr(), b["vs"].data_ptr(), b["ks"].data_ptr(), t_tile.data_ptr(),
                            t_tile.numel(), st)
    if rc:
        raise RuntimeError("reference ES tile sort failed (%d)" % rc)
    torch.cuda.synchronize()
    b["m"] = m
    return b

