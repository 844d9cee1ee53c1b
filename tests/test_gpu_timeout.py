"""Bounded device waits that run out are reported, and leave the GPU usable.

The radix sort's look-back spins on entries that earlier tiles publish.  The
failure-detection hooks make that wait run out without faulting anything:
gsr_debug_stall_sort(1) leaves tile 0 of the first digit pass untaken, so no
one publishes its entry, and gsr_debug_set_sort_wait_limit() shortens the
spin so the tiles after it give up at once.  The sort must then report
GSR_TIMEOUT through the workspace status word, write nothing outside its
buffers, and the next sort (hooks off) must be correct again.
"""
import ctypes

import numpy as np
import pytest
import torch

from polysplat_gb300._lib import GSR_OK, GSR_TIMEOUT, lib

from helpers import random_tile_keys

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stalled(L):
    """Context: every sort launched inside stalls its first pass and gives up fast."""

    class _Ctx:
        def __enter__(self):
            assert L.gsr_debug_set_sort_wait_limit(64) == GSR_OK
            assert L.gsr_debug_stall_sort(1) == GSR_OK

        def __exit__(self, *exc):
            L.gsr_debug_stall_sort(0)
            L.gsr_debug_set_sort_wait_limit(0)
            return False

    return _Ctx()


def test_sort_lookback_timeout_is_reported(cuda_device):
    L = lib()
    rng = np.random.default_rng(11)
    n, end_bit = 100_003, 45
    keys = random_tile_keys(rng, n, (1 << 13) - 1)
    vals = rng.permutation(n).astype(np.uint32)
    ku = torch.from_numpy(keys.view(np.int64).copy()).to(cuda_device)
    vu = torch.from_numpy(vals.view(np.int32).copy()).to(cuda_device)
    # guard words on both sides of the outputs: nothing may be written there
    ks_all = torch.full((n + 2,), 0x5A5A5A5A5A5A5A5A, dtype=torch.int64, device=cuda_device)
    vs_all = torch.full((n + 2,), 0x5A5A5A5A, dtype=torch.int32, device=cuda_device)
    ks, vs = ks_all[1:-1], vs_all[1:-1]
    ws = torch.zeros(L.gsr_workspace_size(n), dtype=torch.int8, device=cuda_device)
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda_device).cuda_stream)
    num = ctypes.c_int32(0)
    with _stalled(L):
        assert L.gsr_sort_bits(n, None, end_bit, _ptr(ws), ws.numel(), _ptr(ku), _ptr(vu), _ptr(ks), _ptr(vs), n,
                               stream) == GSR_OK
        assert L.gsr_read_status(_ptr(ws), None, n, ctypes.byref(num), stream) == GSR_TIMEOUT
    for t, g in ((ks_all, 0x5A5A5A5A5A5A5A5A), (vs_all, 0x5A5A5A5A)):
        assert int(t[0]) == g and int(t[-1]) == g
    # the context is still usable and the same call now sorts correctly
    assert L.gsr_workspace_reset(_ptr(ws), stream) == GSR_OK
    assert L.gsr_sort_bits(n, None, end_bit, _ptr(ws), ws.numel(), _ptr(ku), _ptr(vu), _ptr(ks), _ptr(vs), n,
                           stream) == GSR_OK
    assert L.gsr_read_status(_ptr(ws), None, n, ctypes.byref(num), stream) == GSR_OK
    mask = np.uint64((1 << end_bit) - 1)
    order = np.argsort(keys & mask, kind="stable")
    assert np.array_equal(ks.cpu().numpy().view(np.uint64), keys[order])
    assert np.array_equal(vs.cpu().numpy().view(np.uint32), vals[order])


def test_static_sort_timeout_is_reported(cuda_device):
    L = lib()
    rng = np.random.default_rng(12)
    n, end_bit = 50_000, 44
    keys = random_tile_keys(rng, n, (1 << 12) - 1)
    ku = torch.from_numpy(keys.view(np.int64).copy()).to(cuda_device)
    vu = torch.arange(n, dtype=torch.int32, device=cuda_device)
    ks, vs = torch.empty_like(ku), torch.empty_like(vu)
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda_device).cuda_stream)
    with _stalled(L):
        assert L.gsr_sort_bits_static(n, None, end_bit, _ptr(ku), _ptr(vu), _ptr(ks), _ptr(vs), n, stream) == GSR_OK
        assert L.gsr_sort_bits_static_status(stream) == GSR_TIMEOUT
    assert L.gsr_sort_bits_static(n, None, end_bit, _ptr(ku), _ptr(vu), _ptr(ks), _ptr(vs), n, stream) == GSR_OK
    assert L.gsr_sort_bits_static_status(stream) == GSR_OK
    order = np.argsort(keys & np.uint64((1 << end_bit) - 1), kind="stable")
    assert np.array_equal(ks.cpu().numpy().view(np.uint64), keys[order])
