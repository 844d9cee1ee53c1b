// Depth-first forward pipeline for sm_103a.
//
// The reference orders a frame's (tile, Gaussian) pairs by one radix sort of
// 64-bit tile|depth keys (csrc/cuda_rasterizer/sort.cu:107-125), i.e. it
// orders every pair by depth.  Its "early sorting" mode (preprocess.cu:673-
// 1248, sort.cu:151-285) instead sorts the Gaussians by depth once and emits
// the pairs in that order, after which a stable sort by tile alone gives the
// same per-tile depth order.  This file is this library's version of that
// idea, built on its own kernels:
//   1. counting pass (preprocess.cu, COUNT mode): per Gaussian, the number of
//      tiles its keys go to, its depth bits and its exact test geometry;
//   2. k_df_compact: the emitting Gaussians, in index order (single-pass scan
//      with decoupled look-back, deterministic);
//   3. depth sort of those V Gaussians (32-bit radix sort, sort.cu);
//   4. k_df_offsets: where each Gaussian's pairs start, in depth order, and
//      the total pair count M (written to the caller's key counter);
//   5. emission of (tile, Gaussian) pairs at those offsets: one thread per
//      small rectangle, the CTA-wide massive kernel for the queued ones
//      (preprocess.cu, with the counting pass's tile test);
//   6. stable radix sort of the 32-bit tile ids (2 passes at 1080p instead of
//      5 over 12-byte pairs), then tile ranges from the sorted ids.
// Pairs with the same tile and the same depth bits come out in Gaussian
// index order (the reference's order there depends on its atomics).
#include <algorithm>

#include "gsr_internal.h"

namespace gsr {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;

// Exclusive prefix of this tile's total over all earlier tiles (decoupled
// look-back, one value per tile, bounded spin).  Called by thread 0.
__device__ uint32_t tile_lookback(uint32_t* status, int tile, uint32_t total, uint32_t* err)
{
    st_relaxed_u32(status + tile, (tile == 0 ? kFlagPrefix : kFlagAgg) | (total & kValueMask));
    uint32_t excl = 0;
    int j = tile - 1;
    uint32_t spins = 0;
    while (j >= 0) {
        const uint32_t v = ld_relaxed_u32(status + j);
        if ((v & ~kValueMask) == 0u) {
            if (++spins > kSpinLimit) {
                record_error(err, kErrTimeout);
                break;
            }
            __nanosleep(32);
            continue;
        }
        excl += v & kValueMask;
        if (v & kFlagPrefix) break;
        j--;
    }
    if (tile != 0) st_relaxed_u32(status + tile, kFlagPrefix | ((excl + total) & kValueMask));
    return excl;
}

// Block-wide exclusive scan of one value per thread; returns the total too.
__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t* s_warp, uint32_t& total)
{
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t n = __shfl_up_sync(GSR_FULL_MASK, incl, d);
        if (lane >= (unsigned)d) incl += n;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    uint32_t pre = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; w++) {
        const uint32_t s = s_warp[w];
        if (w < (int)warp) pre += s;
        tot += s;
    }
    total = tot;
    __syncthreads();
    return pre + incl - v;
}

struct DfArgs {
    int P;
    const uint32_t* count;
    const uint32_t* dkey;
    uint32_t* ckeys;
    uint32_t* cgids;
    const uint32_t* sgids;
    uint32_t* offsets;
    uint32_t* rank;
    uint32_t* misc;         // [0] V, [1] compact tile counter, [2] offsets tile counter, [3] M
    uint32_t* status_c;     // look-back of the compaction
    uint32_t* status_o;     // look-back of the offsets scan
    int32_t* m_out;         // the caller's key counter
    uint32_t* err;          // workspace status word
};

// (2) the emitting Gaussians in index order with their depth bits
__global__ __launch_bounds__(kScanThreads) void k_df_compact(const DfArgs a)
{
    __shared__ uint32_t s_warp[kScanThreads / 32];
    __shared__ uint32_t s_tile, s_base;
    const int ntiles = (a.P + kScanTile - 1) / kScanTile;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&a.misc[1], 1u);
        __syncthreads();
        const int tile = (int)s_tile;
        if (tile >= ntiles) break;
        const int g0 = tile * kScanTile + threadIdx.x * kScanItems;  // 8 consecutive Gaussians per thread
        uint32_t flags = 0, n = 0;
#pragma unroll
        for (int j = 0; j < kScanItems; j++) {
            const int g = g0 + j;
            if (g < a.P && __ldg(a.count + g) > 0u) {
                flags |= 1u << j;
                n++;
            }
        }
        uint32_t total;
        const uint32_t excl = block_scan(n, s_warp, total);
        if (threadIdx.x == 0) {
            s_base = tile_lookback(a.status_c, tile, total, a.err);
            if (tile == ntiles - 1) a.misc[0] = s_base + total;
        }
        __syncthreads();
        uint32_t pos = s_base + excl;
#pragma unroll
        for (int j = 0; j < kScanItems; j++) {
            if (flags & (1u << j)) {
                a.ckeys[pos] = __ldg(a.dkey + g0 + j);
                a.cgids[pos] = (uint32_t)(g0 + j);
                pos++;
            }
        }
        __syncthreads();
    }
}

// (4) offsets of each depth-ordered Gaussian's pairs; M = their total
__global__ __launch_bounds__(kScanThreads) void k_df_offsets(const DfArgs a)
{
    __shared__ uint32_t s_warp[kScanThreads / 32];
    __shared__ uint32_t s_tile, s_base;
    const int V = (int)min(a.misc[0], (uint32_t)a.P);
    const int ntiles = (V + kScanTile - 1) / kScanTile;
    if (V == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            a.misc[3] = 0u;
            *a.m_out = 0;
        }
        return;
    }
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&a.misc[2], 1u);
        __syncthreads();
        const int tile = (int)s_tile;
        if (tile >= ntiles) break;
        const int s0 = tile * kScanTile + threadIdx.x * kScanItems;
        uint32_t c[kScanItems];
        uint32_t n = 0;
#pragma unroll
        for (int j = 0; j < kScanItems; j++) {
            const int s = s0 + j;
            c[j] = s < V ? __ldg(a.count + __ldg(a.sgids + s)) : 0u;
            n += c[j];
        }
        uint32_t total;
        const uint32_t excl = block_scan(n, s_warp, total);
        if (threadIdx.x == 0) {
            s_base = tile_lookback(a.status_o, tile, total, a.err);
            if (tile == ntiles - 1) {
                const uint32_t m = s_base + total;
                a.misc[3] = m;
                *a.m_out = (int32_t)m;
            }
        }
        __syncthreads();
        uint32_t off = s_base + excl;
#pragma unroll
        for (int j = 0; j < kScanItems; j++) {
            const int s = s0 + j;
            if (s < V) {
                a.offsets[s] = off;
                a.rank[__ldg(a.sgids + s)] = (uint32_t)s;
                off += c[j];
            }
        }
        __syncthreads();
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// Scene scratch layout (per-Gaussian arrays + the depth sort's scratch).

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

size_t df_scratch_bytes(int P)
{
    const size_t p = (size_t)(P < 1 ? 1 : P);
    const size_t tiles = (p + kScanTile - 1) / kScanTile;
    return 256 + al(p * 4) * 8 + al(p * 16) + al(p * 8) + 2 * al(tiles * 4) + sort_scratch_bytes((long long)p, 4);
}

struct DfLayout {
    uint32_t *misc, *count, *dkey, *rank, *ckeys, *cgids, *skeys, *sgids, *offsets, *status_c, *status_o;
    float4* geo;
    int2* rect;
    void* sort_mem;
    size_t status_bytes;
};

static DfLayout df_layout(void* scratch, int P)
{
    const size_t p = (size_t)(P < 1 ? 1 : P);
    const size_t tiles = (p + kScanTile - 1) / kScanTile;
    char* b = reinterpret_cast<char*>(scratch);
    DfLayout L;
    size_t o = 0;
    L.misc = reinterpret_cast<uint32_t*>(b + o);
    o += 256;
    uint32_t** arr[8] = {&L.count, &L.dkey, &L.rank, &L.ckeys, &L.cgids, &L.skeys, &L.sgids, &L.offsets};
    for (auto q : arr) {
        *q = reinterpret_cast<uint32_t*>(b + o);
        o += al(p * 4);
    }
    L.geo = reinterpret_cast<float4*>(b + o);
    o += al(p * 16);
    L.rect = reinterpret_cast<int2*>(b + o);
    o += al(p * 8);
    L.status_c = reinterpret_cast<uint32_t*>(b + o);
    L.status_o = reinterpret_cast<uint32_t*>(b + o + al(tiles * 4));
    L.status_bytes = 2 * al(tiles * 4);
    o += L.status_bytes;
    L.sort_mem = b + o;
    return L;
}

cudaError_t launch_depth_first(const PreprocessParams& p0, bool half_sh, void* scratch, size_t scratch_bytes,
                               WorkspaceHeader* hdr, const SortScratch& tile_sort, int tiles, uint32_t* tile_keys_in,
                               uint32_t* vals_in, uint32_t* tile_keys_out, uint32_t* vals_out, int2* ranges,
                               cudaStream_t stream)
{
    if (scratch_bytes < df_scratch_bytes(p0.P)) return cudaErrorInvalidValue;
    const DfLayout L = df_layout(scratch, p0.P);
    PreprocessParams p = p0;
    p.df.count = L.count;
    p.df.dkey = L.dkey;
    p.df.geo = L.geo;
    p.df.rect = L.rect;

    cudaError_t e = launch_preprocess_count(p, half_sh, stream);
    if (e != cudaSuccess) return e;
    profile_mark(stream);

    // clear the scan counters / look-back state (misc + both status arrays)
    if ((e = cudaMemsetAsync(L.misc, 0, 256, stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(L.status_c, 0, L.status_bytes, stream)) != cudaSuccess) return e;
    if (p.P > 0) {
        DfArgs a;
        a.P = p.P;
        a.count = L.count;
        a.dkey = L.dkey;
        a.ckeys = L.ckeys;
        a.cgids = L.cgids;
        a.sgids = L.sgids;
        a.offsets = L.offsets;
        a.rank = L.rank;
        a.misc = L.misc;
        a.status_c = L.status_c;
        a.status_o = L.status_o;
        a.m_out = p.counter;
        a.err = &hdr->status;
        const int sms = device_sm_count();
        const int ntiles = div_up(p.P, kScanTile);
        k_df_compact<<<std::min(ntiles, sms * 4), kScanThreads, 0, stream>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        profile_mark(stream);

        // depth sort of the V emitting Gaussians (count read on the device)
        const SortScratch ds = carve_sort_scratch(hdr, L.sort_mem, p.P, 4);
        OrderMap od{kOrderDepth32, 32};
        e = launch_sort32(0, reinterpret_cast<const int32_t*>(&L.misc[0]), p.P, od, 4, L.ckeys, L.cgids, L.skeys,
                          L.sgids, ds, stream);
        if (e != cudaSuccess) return e;

        k_df_offsets<<<std::min(ntiles, sms * 4), kScanThreads, 0, stream>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        profile_mark(stream);
        e = launch_df_emit_small(p, &L.misc[0], L.sgids, L.offsets, tile_keys_in, vals_in, p.cap, stream);
        if (e != cudaSuccess) return e;
        e = launch_df_emit_massive(p, L.offsets, L.rank, tile_keys_in, vals_in, p.cap, stream);
        if (e != cudaSuccess) return e;
        profile_mark(stream);
    } else {
        if ((e = cudaMemsetAsync(p.counter, 0, sizeof(int32_t), stream)) != cudaSuccess) return e;
    }

    // stable sort of the tile ids (M read on the device)
    const int tb = bits_for((uint32_t)tiles);
    OrderMap ot{kOrderMasked, tb, 0};  // tile ids
    e = launch_sort32(0, p.counter, p.cap, ot, (tb + 7) / 8, tile_keys_in, vals_in, tile_keys_out, vals_out, tile_sort,
                      stream);
    if (e != cudaSuccess) return e;
    e = launch_tile_ranges32(p.counter, p.cap, tiles, tile_keys_out, ranges, stream);
    if (e != cudaSuccess) return e;
    profile_mark(stream);
    return cudaSuccess;
}

}  // namespace gsr
