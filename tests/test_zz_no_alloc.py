"""The static-scratch sort entry point (gsr_sort_bits_static) against the
workspace sort (gsr_sort_bits), through the C ABI.

Collected last on purpose: it must pass both after every other test in the
same process and alone in a fresh process (the first call on a device looks
up the scratch address).  Integer sort, so the bar is bit-exact, on two calls
in a row into fresh outputs.
"""
import ctypes

import numpy as np
import pytest
import torch

from polysplat_gb300._lib import GSR_INVALID_ARG, GSR_OK, lib

from helpers import random_tile_keys

pytestmark = pytest.mark.gpu

STATIC_MAX = 1 << 18


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("n,end_bit", [(1, 45), (4097, 43), (200_003, 45), (STATIC_MAX, 49)])
def test_static_sort_matches_workspace_sort(cuda_device, n, end_bit):
    L = lib()
    rng = np.random.default_rng(n + end_bit)
    tiles = (1 << (end_bit - 32)) - 1
    keys = random_tile_keys(rng, n, tiles, high_garbage=True, end_bit=end_bit)
    vals = rng.permutation(n).astype(np.uint32)
    ku = torch.from_numpy(keys.view(np.int64).copy()).to(cuda_device)
    vu = torch.from_numpy(vals.view(np.int32).copy()).to(cuda_device)
    ks_ref, vs_ref = torch.empty_like(ku), torch.empty_like(vu)
    ws = torch.zeros(L.gsr_workspace_size(n), dtype=torch.int8, device=cuda_device)
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda_device).cuda_stream)
    assert L.gsr_sort_bits(n, None, end_bit, _ptr(ws), ws.numel(), _ptr(ku), _ptr(vu), _ptr(ks_ref), _ptr(vs_ref), n,
                           stream) == GSR_OK
    outs = [(torch.full_like(ku, -1), torch.full_like(vu, -1)) for _ in range(2)]
    free, reserved = [], []
    for ks, vs in outs:  # two calls in a row
        assert L.gsr_sort_bits_static(n, None, end_bit, _ptr(ku), _ptr(vu), _ptr(ks), _ptr(vs), n, stream) == GSR_OK
        assert L.gsr_sort_bits_static_status(stream) == GSR_OK
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info(cuda_device)[0])
        reserved.append(torch.cuda.memory_reserved(cuda_device))
    # the scratch array comes with the library's device code (loaded, with
    # lazy module loading, by the first call); a call itself allocates nothing
    assert reserved[1] == reserved[0], "torch's caching allocator grew between the calls"
    assert free[1] == free[0], (
        "device free memory changed between two static sorts (%d -> %d bytes) while torch's reserve stayed the "
        "same: either the entry point allocated, or another context on this GPU did" % (free[0], free[1]))
    for ks, vs in outs:
        assert torch.equal(ks, ks_ref) and torch.equal(vs, vs_ref)


def test_static_sort_device_count(cuda_device):
    L = lib()
    rng = np.random.default_rng(5)
    n, cap, end_bit = 70_000, 100_000, 45
    keys = random_tile_keys(rng, cap, (1 << 13) - 1)
    ku = torch.from_numpy(keys.view(np.int64).copy()).to(cuda_device)
    vu = torch.arange(cap, dtype=torch.int32, device=cuda_device)
    d_num = torch.tensor([n], dtype=torch.int32, device=cuda_device)
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda_device).cuda_stream)
    ks_ref, vs_ref = torch.full_like(ku, -1), torch.full_like(vu, -1)
    ws = torch.zeros(L.gsr_workspace_size(cap), dtype=torch.int8, device=cuda_device)
    assert L.gsr_sort_bits(0, _ptr(d_num), end_bit, _ptr(ws), ws.numel(), _ptr(ku), _ptr(vu), _ptr(ks_ref),
                           _ptr(vs_ref), cap, stream) == GSR_OK
    for _ in range(2):
        ks, vs = torch.full_like(ku, -1), torch.full_like(vu, -1)
        assert L.gsr_sort_bits_static(0, _ptr(d_num), end_bit, _ptr(ku), _ptr(vu), _ptr(ks), _ptr(vs), cap,
                                      stream) == GSR_OK
        assert L.gsr_sort_bits_static_status(stream) == GSR_OK
        torch.cuda.synchronize()
        assert torch.equal(ks[:n], ks_ref[:n]) and torch.equal(vs[:n], vs_ref[:n])


def test_static_sort_rejects_capacity_beyond_its_scratch(cuda_device):
    L = lib()
    n = STATIC_MAX + 1
    ku = torch.zeros(n, dtype=torch.int64, device=cuda_device)
    vu = torch.zeros(n, dtype=torch.int32, device=cuda_device)
    ks, vs = torch.empty_like(ku), torch.empty_like(vu)
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda_device).cuda_stream)
    assert L.gsr_sort_bits_static(n, None, 45, _ptr(ku), _ptr(vu), _ptr(ks), _ptr(vs), n, stream) == GSR_INVALID_ARG
