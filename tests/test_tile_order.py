"""Tile-order helpers (render.cu:4414-4866, 6959-7087): the numpy oracle on
known answers, and the library's kernels against the oracle on the GPU
(bit-exact: order, sorted keys, ids and descriptors)."""
import numpy as np
import pytest
import torch

from oracle import oracle as ora


def test_oracle_tile_order_known_answers():
    ranges = np.array([[0, 3], [3, 4], [4, 7], [7, 7], [7, 12]], np.int32)  # counts 3 1 3 0 5
    order, keys, ids, desc = ora.tile_order(ranges, x_blocks=5)
    assert order.tolist() == [4, 0, 2, 1, 3]  # descending, equal counts in index order
    assert keys.tolist() == [5, 3, 3, 1, 0]
    assert ids.tolist() == [0, 1, 2, 3, 4]
    assert desc.tolist() == [[4, 0, 7, 12], [0, 0, 0, 3], [2, 0, 4, 7], [1, 0, 3, 4], [3, 0, 7, 7]]
    # zig-zag over groups of 2: group 1 (positions 2, 3) reads the order
    # backwards; groups 0 and 2 read it forwards
    _, _, _, dz = ora.tile_order(ranges, x_blocks=5, zigzag=2)
    assert dz[:, 0].tolist() == [4, 0, 1, 2, 3]
    # Morton key on a 2x2 grid, bucket 4: counts 3 1 3 0 -> bucket 0 for all;
    # Morton codes (0,0)=0 (1,0)=1 (0,1)=2 (1,1)=3, so ascending Morton order
    r4 = ranges[:4]
    o4, k4, _, _ = ora.tile_order(r4, x_blocks=2, morton_bucket=4)
    assert o4.tolist() == [0, 1, 2, 3]
    assert k4.tolist() == [0xFFFF, 0xFFFE, 0xFFFD, 0xFFFC]
    # bucket 2: counts 3 1 3 0 -> buckets 1 0 1 0
    o2, _, _, _ = ora.tile_order(r4, x_blocks=2, morton_bucket=2)
    assert o2.tolist() == [0, 2, 1, 3]


def _ranges(T, seed):
    rng = np.random.default_rng(seed)
    counts = rng.integers(0, 6, T)  # many ties
    big = rng.random(T) < 0.05
    counts[big] = rng.integers(100, 20_000, int(big.sum()))
    counts[rng.random(T) < 0.2] = 0
    ends = np.cumsum(counts)
    return np.stack([ends - counts, ends], axis=1).astype(np.int32)


@pytest.mark.gpu
@pytest.mark.parametrize("W,H", [(800, 600), (1920, 1080), (7680, 4320)])
@pytest.mark.parametrize("morton,zigzag", [(0, 0), (0, 152), (64, 0), (16, 7)])
def test_tile_order_matches_oracle(cuda_device, W, H, morton, zigzag):
    from polysplat_gb300 import ops
    gx, gy = (W + 15) // 16, (H + 15) // 16
    T = gx * gy
    rn = _ranges(T, seed=T + morton + zigzag)
    dev = cuda_device
    ranges = torch.from_numpy(rn).to(dev)
    order = torch.full((T,), -1, dtype=torch.int32, device=dev)
    counts = torch.full((T,), -1, dtype=torch.int32, device=dev)
    ids = torch.full((T,), -1, dtype=torch.int32, device=dev)
    desc = torch.full((T, 4), -1, dtype=torch.int32, device=dev)
    temp = torch.zeros(ops.get_tile_order_sort_temp_size(T), dtype=torch.int8, device=dev)
    if morton:
        ops.compute_tile_order_packed_morton(ranges, T, gx, desc, order, counts, ids, temp, zigzag, morton)
    else:
        ops.compute_tile_order_packed(ranges, T, gx, desc, order, counts, ids, temp, zigzag)
    torch.cuda.synchronize()
    o, k, i, d = ora.tile_order(rn, gx, morton, zigzag)
    assert np.array_equal(order.cpu().numpy().view(np.uint32), o)
    assert np.array_equal(counts.cpu().numpy().view(np.uint32), k)
    assert np.array_equal(ids.cpu().numpy().view(np.uint32), i)
    assert np.array_equal(desc.cpu().numpy(), d)
    if morton == 0 and zigzag == 0:
        order2 = torch.full((T,), -1, dtype=torch.int32, device=dev)
        ops.compute_tile_order(ranges, T, order2, counts, ids, temp)
        torch.cuda.synchronize()
        assert np.array_equal(order2.cpu().numpy().view(np.uint32), o)
        back = ops._desc_to_ranges(desc, W, H)
        assert np.array_equal(back.cpu().numpy(), rn)
