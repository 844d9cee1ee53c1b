"""ctypes binding of ``libgsr.so`` (the C ABI declared in ``include/gsr.h``).

The library is built in-tree by :mod:`polysplat_gb300.build`.  There is no
fallback: if the shared library is missing or no GB300 is present, every
entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

GSR_OK, GSR_OVERFLOW, GSR_TIMEOUT, GSR_INVALID_ARG, GSR_CUDA_ERROR = range(5)
STATUS_NAMES = {0: "OK", 1: "OVERFLOW", 2: "TIMEOUT", 3: "INVALID_ARG", 4: "CUDA_ERROR"}

RENDER_PERSISTENT_RANGES = 0
RENDER_PERSISTENT_FUSED = 1
RENDER_DEFAULT = 2
RENDER_RANGES_CADENCE2 = 3
RENDER_DT = 4
RENDER_SPLIT = 5
QUAD_KEYS = 0x100  # GSR_QUAD_KEYS: one key per 2x2 group of 16x16 tiles


class GsrError(RuntimeError):
    def __init__(self, status: int, where: str, num: int = -1):
        self.status = status
        self.num = num
        msg = "gsr %s failed: %s" % (where, STATUS_NAMES.get(status, str(status)))
        if status == GSR_OVERFLOW:
            msg += " (%d keys emitted; the key buffers are too small)" % num
        if status == GSR_CUDA_ERROR and _lib is not None:
            msg += " (%s)" % _lib.gsr_last_error().decode(errors="replace")
        super().__init__(msg)


def _declare(L):
    P, i32, i64, f32, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_size_t
    sig = {
        "gsr_version": ([], i32),
        "gsr_device_check": ([i32], i32),
        "gsr_workspace_size": ([i64], sz),
        "gsr_render_workspace_size": ([], sz),
        "gsr_workspace_reset": ([P, P], i32),
        "gsr_read_status": ([P, P, i64, P, P], i32),
        "gsr_scene_prepare": ([i32, P, P, P, P, P, P], i32),
        "gsr_preprocess": ([i32, P, P, i32, P, P, i32, i32, i32, i32, P, P, f32, f32, f32, f32,
                            P, P, P, P, P, i64, P, P, sz, P], i32),
        "gsr_sort": ([i32, P, i32, i32, i32, i32, P, sz, P, P, P, P, i64, P], i32),
        "gsr_sort_bits": ([i32, P, i32, P, sz, P, P, P, P, i64, P], i32),
        "gsr_tile_ranges": ([i32, P, i32, i32, i32, i32, P, P, i32, P], i32),
        "gsr_gather": ([i32, P, P, P, P, P, P, P, P, P], i32),
        "gsr_render": ([i32, i32, P, i32, i32, i32, i32, i32, P, P, P, P, P, P, P, P, P, P], i32),
        "gsr_forward": ([i32, i32, P, P, i32, P, P, i32, i32, i32, i32, P, P, f32, f32, f32, f32,
                         P, P, sz, P, P, P, P, i64, P, P, P, P, P, P, P], i32),
    }
    sig["gsr_sort_bits_static"] = ([i32, P, i32, P, P, P, P, i64, P], i32)
    sig["gsr_sort_bits_static_status"] = ([P], i32)
    sig["gsr_debug_set_sort_wait_limit"] = ([ctypes.c_uint32], i32)
    sig["gsr_debug_stall_sort"] = ([i32], i32)
    sig["gsr_batcher_device_bytes"] = ([i32, i64, i64, i32], sz)
    sig["gsr_batcher_create"] = ([i32, i64, i64, i32], P)
    sig["gsr_batcher_destroy"] = ([P], None)
    sig["gsr_batcher_render"] = ([P, i32, i32, i32, i32, P, i32, P, i32, i32, P], i32)
    sig["gsr_batcher_finish"] = ([P, P, P], i32)
    sig["gsr_batcher_graphs"] = ([P], i32)
    sig["gsr_batcher_set_thresholds"] = ([P, i32, i32], i32)
    sig["gsr_batcher_counter"] = ([P], P)
    sig["gsr_batcher_status"] = ([P], P)
    sig["gsr_train_forward"] = ([i32, P, P, P, P, P, i32, i32, P, P, f32, f32, f32, f32, P, P, P, P, P, sz,
                                 P, P, P, P, i64, P, P, P, P, P, P, P, P], i32)
    sig["gsr_train_backward"] = ([i32, P, P, P, P, P, i32, i32, P, P, f32, f32, f32, f32, P, P, i64, P, P, P, P,
                                  P, P, P, P, P, P, P, P, P, P, P, P, i32, P], i32)
    sig["gsr_train_views_scratch_bytes"] = ([i32], sz)
    sig["gsr_train_forward_views"] = ([i32, P, P, P, P, P, i32, i32, i32, P, P, P, P, P, P, P, sz, P, P, sz,
                                       P, P, P, P, i64, P, P, P, P, P, P, P, i32, P], i32)
    sig["gsr_train_backward_views"] = ([i32, P, P, P, P, P, i32, i32, i32, P, P, P, P, P, i64, P, P, P, P,
                                        P, P, P, P, P, P, P, P, P, P, i32, i32, P], i32)
    sig["gsr_depth_first_scratch_size"] = ([i32], sz)
    sig["gsr_forward_depth_first"] = ([i32, i32, P, P, i32, P, P, i32, i32, i32, i32, P, P, f32, f32, f32, f32,
                                       P, P, sz, P, sz, P, P, P, P, i64, P, P, P, P, P, P, P], i32)
    sig["gsr_es_pass_a"] = ([i32, P, P, i32, P, P, i32, i32, i32, i32, P, P, f32, f32, f32, f32,
                             P, P, P, P, P, P, P, P], i32)
    sig["gsr_es_scan_buffer_size"] = ([i32], sz)
    sig["gsr_es_depth_sort_and_scan"] = ([i32, P, P, P, P, P, P, P, P, P, sz, P, sz, P], i32)
    sig["gsr_es_pass_b"] = ([i32, i32, i32, i32, i32, P, P, P, P, P, P, P, P, i64, P], i32)
    sig["gsr_es_tile_sort"] = ([i32, i32, i32, i32, i32, P, P, P, P, P, P, sz, P], i32)
    sig["gsr_tile_order_temp_size"] = ([i32], sz)
    sig["gsr_tile_order"] = ([P, i32, i32, i32, i32, P, P, P, P, P, sz, P], i32)
    sig["gsr_tile_desc_ranges"] = ([P, i32, i32, P, P], i32)
    sig["gsr_camera_matrices"] = ([i32, i32, P, P, f32, f32, f32, f32, P, P], None)
    sig["gsr_profile_begin"] = ([i32], i32)
    sig["gsr_profile_read"] = ([P, i32, i32], i32)
    sig["gsr_profile_end"] = ([], None)
    sig["gsr_last_error"] = ([], ctypes.c_char_p)
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    return L


def lib():
    """Load (building first if needed) the gsr shared library."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                path = _build.LIB
                if not os.path.exists(path) or os.environ.get("GSR_REBUILD"):
                    path = _build.build()
                _lib = _declare(ctypes.CDLL(path))
    return _lib


def check(status: int, where: str, num: int = -1) -> None:
    if status != GSR_OK:
        raise GsrError(status, where, num)
