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
//   2. k_df_compact: the emitting Gaussians, in index order (reduce-then-scan,
//      deterministic);
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
    uint32_t* misc;         // [0] V, [3] M
    uint32_t* sums_c;       // per-tile counts of emitting Gaussians, then their exclusive scan
    uint32_t* sums_o;       // per-tile pair counts in depth order, then their exclusive scan
    uint32_t* csorted;      // the pair counts in depth order
    int32_t* m_out;         // the caller's key counter
    uint32_t* err;          // workspace status word
};

// Both scans are reduce-then-scan: per-tile sums, one CTA scans the sums, and
// each tile then scans itself from its base.  (A single pass with decoupled
// look-back stalls here: with hundreds of CTAs in flight every tile walks
// back over hundreds of unfinished predecessors.)

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* s_warp)
{
    uint32_t total;
    block_scan(v, s_warp, total);
    return total;
}

// (2a) per tile, how many Gaussians emit
__global__ __launch_bounds__(kScanThreads) void k_df_compact_sums(const DfArgs a)
{
    __shared__ uint32_t s_warp[kScanThreads / 32];
    const int ntiles = (a.P + kScanTile - 1) / kScanTile;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        uint32_t n = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            const int g = tile * kScanTile + k * kScanThreads + (int)threadIdx.x;
            n += (g < a.P && __ldg(a.count + g) > 0u) ? 1u : 0u;
        }
        const uint32_t t = block_sum(n, s_warp);
        if (threadIdx.x == 0) a.sums_c[tile] = t;
    }
}

// (2b, 4b) exclusive scan of `n` tile sums in place by one CTA; the total goes
// to misc[slot] (and, for the pair count, to the caller's key counter)
__global__ __launch_bounds__(1024) void k_df_scan_sums(const uint32_t* d_n_elems, int n_max_elems, uint32_t* sums,
                                                       uint32_t* misc, int slot, int32_t* m_out)
{
    __shared__ uint32_t s_w[32];
    const int elems = d_n_elems ? (int)min(*d_n_elems, (uint32_t)n_max_elems) : n_max_elems;
    const int nb = (elems + kScanTile - 1) / kScanTile;
    const int per = (nb + 1023) / 1024, j0 = (int)threadIdx.x * per;
    uint32_t v = 0;
    for (int j = j0; j < min(nb, j0 + per); j++) v += sums[j];
    uint32_t incl = v;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(GSR_FULL_MASK, incl, d);
        if (lane >= (unsigned)d) incl += t;
    }
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    uint32_t wpre = 0, all = 0;
    for (int w = 0; w < 32; w++) {
        if (w < (int)warp) wpre += s_w[w];
        all += s_w[w];
    }
    uint32_t run = wpre + incl - v;
    for (int j = j0; j < min(nb, j0 + per); j++) {
        const uint32_t c = sums[j];
        sums[j] = run;
        run += c;
    }
    if (threadIdx.x == 0) {
        misc[slot] = all;
        if (m_out) *m_out = (int32_t)all;
    }
}

// (2c) the emitting Gaussians in index order with their depth bits
__global__ __launch_bounds__(kScanThreads) void k_df_compact(const DfArgs a)
{
    __shared__ uint32_t s_warp[kScanThreads / 32];
    const int ntiles = (a.P + kScanTile - 1) / kScanTile;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
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
        uint32_t pos = a.sums_c[tile] + block_scan(n, s_warp, total);
#pragma unroll
        for (int j = 0; j < kScanItems; j++) {
            if (flags & (1u << j)) {
                a.ckeys[pos] = __ldg(a.dkey + g0 + j);
                a.cgids[pos] = (uint32_t)(g0 + j);
                pos++;
            }
        }
    }
}

// (4a) the pair counts in depth order, and their per-tile sums
__global__ __launch_bounds__(kScanThreads) void k_df_offsets_sums(const DfArgs a)
{
    __shared__ uint32_t s_warp[kScanThreads / 32];
    const int V = (int)min(a.misc[0], (uint32_t)a.P);
    const int ntiles = (V + kScanTile - 1) / kScanTile;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        uint32_t n = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            const int sidx = tile * kScanTile + k * kScanThreads + (int)threadIdx.x;
            if (sidx < V) {
                const uint32_t gid = __ldg(a.sgids + sidx);
                const uint32_t c = gid < (uint32_t)a.P ? __ldg(a.count + gid) : 0u;
                a.csorted[sidx] = c;
                n += c;
            }
        }
        const uint32_t t = block_sum(n, s_warp);
        if (threadIdx.x == 0) a.sums_o[tile] = t;
    }
}

// (4c) where each Gaussian's pairs start, in depth order, and its rank
__global__ __launch_bounds__(kScanThreads) void k_df_offsets(const DfArgs a)
{
    __shared__ uint32_t s_warp[kScanThreads / 32];
    const int V = (int)min(a.misc[0], (uint32_t)a.P);
    const int ntiles = (V + kScanTile - 1) / kScanTile;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int s0 = tile * kScanTile + threadIdx.x * kScanItems;
        uint32_t c[kScanItems];
        uint32_t n = 0;
#pragma unroll
        for (int j = 0; j < kScanItems; j++) {
            c[j] = s0 + j < V ? __ldg(a.csorted + s0 + j) : 0u;
            n += c[j];
        }
        uint32_t total;
        uint32_t off = a.sums_o[tile] + block_scan(n, s_warp, total);
#pragma unroll
        for (int j = 0; j < kScanItems; j++) {
            const int sidx = s0 + j;
            if (sidx < V) {
                a.offsets[sidx] = off;
                const uint32_t gid = __ldg(a.sgids + sidx);
                if (gid < (uint32_t)a.P) a.rank[gid] = (uint32_t)sidx;
                off += c[j];
            }
        }
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
    uint32_t *misc, *count, *dkey, *rank, *ckeys, *cgids, *skeys, *sgids, *offsets, *sums_c, *sums_o;
    float4* geo;
    int2* rect;
    void* sort_mem;
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
    L.sums_c = reinterpret_cast<uint32_t*>(b + o);
    L.sums_o = reinterpret_cast<uint32_t*>(b + o + al(tiles * 4));
    o += 2 * al(tiles * 4);
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

    if ((e = cudaMemsetAsync(L.misc, 0, 256, stream)) != cudaSuccess) return e;
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
        a.sums_c = L.sums_c;
        a.sums_o = L.sums_o;
        a.csorted = L.skeys;  // the sorted depth keys are not read after the depth sort
        a.m_out = p.counter;
        a.err = &hdr->status;
        const int sms = device_sm_count();
        const int grid = std::min(div_up(p.P, kScanTile), sms * 8);
        k_df_compact_sums<<<grid, kScanThreads, 0, stream>>>(a);
        k_df_scan_sums<<<1, 1024, 0, stream>>>(nullptr, p.P, L.sums_c, L.misc, 0, nullptr);
        k_df_compact<<<grid, kScanThreads, 0, stream>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        profile_mark(stream);

        // depth sort of the V emitting Gaussians (count read on the device)
        const SortScratch ds = carve_sort_scratch(hdr, L.sort_mem, p.P, 4);
        OrderMap od{kOrderDepth32, 32};
        e = launch_sort32(0, reinterpret_cast<const int32_t*>(&L.misc[0]), p.P, od, 4, L.ckeys, L.cgids, L.skeys,
                          L.sgids, ds, stream);
        if (e != cudaSuccess) return e;

        k_df_offsets_sums<<<grid, kScanThreads, 0, stream>>>(a);
        k_df_scan_sums<<<1, 1024, 0, stream>>>(&L.misc[0], p.P, L.sums_o, L.misc, 3, p.counter);
        k_df_offsets<<<grid, kScanThreads, 0, stream>>>(a);
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
