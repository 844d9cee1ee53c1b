"""Shared helpers of the parity tests."""
import math

import numpy as np


def psnr(a: np.ndarray, b: np.ndarray) -> float:
    d = a.astype(np.float64) - b.astype(np.float64)
    mse = float(np.mean(d * d))
    return float("inf") if mse == 0 else 10.0 * math.log10(255.0 ** 2 / mse)


def image_stats(a, b):
    d = np.abs(a.astype(np.int32) - b.astype(np.int32))
    return dict(max_abs=int(d.max()) if d.size else 0, psnr=psnr(a, b), frac_diff=float((d > 0).mean()))


def key_pairs(keys: np.ndarray, vals: np.ndarray):
    """(tile, gaussian) pair set and the depth bits per pair."""
    t = (keys >> np.uint64(32)).astype(np.int64)
    d = (keys & np.uint64(0xFFFFFFFF)).astype(np.int64)
    pair = t * (1 << 32) + vals.astype(np.int64)
    order = np.argsort(pair, kind="stable")
    return pair[order], d[order]


def compare_key_lists(gk, gv, ok, ov):
    """Return (n_only_gpu, n_only_oracle, max_depth_ulp over common pairs)."""
    gp, gd = key_pairs(gk, gv)
    op, od = key_pairs(ok, ov)
    common, gi, oi = np.intersect1d(gp, op, assume_unique=False, return_indices=True)
    only_g = gp.size - common.size
    only_o = op.size - common.size
    ulp = int(np.abs(gd[gi] - od[oi]).max()) if common.size else 0
    return only_g, only_o, ulp


def random_tile_keys(rng, n, tiles, dup_frac=0.2, high_garbage=False, end_bit=64):
    t = rng.integers(0, max(1, tiles), n).astype(np.uint64)
    d = rng.uniform(0.2, 60.0, n).astype(np.float32).view(np.uint32).astype(np.uint64)
    if n and dup_frac:
        k = int(n * dup_frac)
        d[:k] = d[0]
    keys = (t << np.uint64(32)) | d
    if high_garbage and end_bit < 64:
        g = rng.integers(0, 2, n).astype(np.uint64) << np.uint64(end_bit)
        keys |= g
    return keys
