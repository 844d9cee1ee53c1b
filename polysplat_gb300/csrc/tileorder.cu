// Tile-order helpers of the reference's reordered renders (render.cu:4414-4535,
// 4813-4866, 6959-7087): tiles sorted by descending key count (stable), or by
// a (count bucket, Morton position) composite key, and packed tile
// descriptors {col, row, start, end} in that order, optionally zig-zagged
// over groups.  The descending sort is this library's ascending radix sort
// of the complemented keys (complementing keeps equal keys in index order).
#include <algorithm>

#include "gsr_internal.h"

namespace gsr {
namespace {

__device__ __forceinline__ uint32_t spread_bits16(uint32_t v)
{
    v &= 0xFFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

// complemented sort keys and tile ids; morton_bucket > 0 selects the
// composite key (min(count / bucket, 0xFFFF) << 16) | (0xFFFF - morton & 0xFFFF)
__global__ void k_tile_keys(const int2* __restrict__ ranges, int T, int x_blocks, int morton_bucket,
                            uint32_t* __restrict__ keys_c, uint32_t* __restrict__ ids)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) {
        const int2 r = ranges[t];
        uint32_t key = (uint32_t)(r.y - r.x);
        if (morton_bucket > 0) {
            const uint32_t bucket = min(key / (uint32_t)morton_bucket, 0xFFFFu);
            const uint32_t x = (uint32_t)(t % x_blocks), y = (uint32_t)(t / x_blocks);
            const uint32_t morton = (spread_bits16(x) | (spread_bits16(y) << 1)) & 0xFFFFu;
            key = (bucket << 16) | (0xFFFFu - morton);
        }
        keys_c[t] = ~key;
        ids[t] = (uint32_t)t;
    }
}

// undo the complement of the sorted keys; with desc != nullptr also write the
// descriptor of every position (zig-zag over groups of `group` when group > 1:
// odd groups read their slice of the order backwards)
__global__ void k_tile_desc(uint32_t* __restrict__ sorted_c, const uint32_t* __restrict__ order,
                            const int2* __restrict__ ranges, int T, int x_blocks, int group, int4* __restrict__ desc)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < T; i += gridDim.x * blockDim.x) {
        sorted_c[i] = ~sorted_c[i];
        if (!desc) continue;
        int src = i;
        if (group > 1) {
            const int g = i / group, base = g * group, len = min(base + group, T) - base;
            src = (g & 1) ? base + (len - 1 - (i - base)) : i;
            src = min(src, T - 1);
        }
        const uint32_t id = order[src];
        int4 d = make_int4((int)(id % (uint32_t)x_blocks), (int)(id / (uint32_t)x_blocks), 0, 0);
        if (id < (uint32_t)T) {
            const int2 r = ranges[id];
            d.z = r.x;
            d.w = r.y;
        }
        desc[i] = d;
    }
}

__global__ void k_desc_ranges(const int4* __restrict__ desc, int T, int x_blocks, int2* __restrict__ ranges)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < T; i += gridDim.x * blockDim.x) {
        const int4 d = desc[i];
        if (d.x < 0 || d.x >= x_blocks || d.y < 0) continue;
        const long long t = (long long)d.y * x_blocks + d.x;
        if (t < T) ranges[t] = make_int2(d.z, d.w);
    }
}

int grid_of(int n) { return std::max(1, std::min(device_sm_count() * 8, (n + 255) / 256)); }

size_t round256(size_t x) { return (x + 255) & ~(size_t)255; }

// temp layout: [header][radix-sort scratch][complemented keys]
size_t keys_offset(int T) { return kHeaderBytes + round256(sort_scratch_bytes(T, 4)); }

}  // namespace
}  // namespace gsr

using namespace gsr;

extern "C" {

size_t gsr_tile_order_temp_size(int total_tiles)
{
    const int T = std::max(1, total_tiles);
    return keys_offset(T) + round256((size_t)T * 4);
}

gsr_status gsr_tile_order(const int32_t* tile_ranges, int total_tiles, int x_blocks, int morton_bucket,
                          int zigzag_group, int32_t* tile_desc, uint32_t* tile_order, uint32_t* tile_counts,
                          uint32_t* tile_ids, void* temp, size_t temp_bytes, gsr_stream_t stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (total_tiles < 0 || x_blocks <= 0 || morton_bucket < 0) return GSR_INVALID_ARG;
    if (total_tiles == 0) return GSR_OK;
    if (!tile_ranges || !tile_order || !tile_counts || !tile_ids || !temp ||
        temp_bytes < gsr_tile_order_temp_size(total_tiles) || total_tiles >= (1 << 30))
        return GSR_INVALID_ARG;
    const int T = total_tiles;
    uint32_t* keys_c = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(temp) + keys_offset(T));
    const SortScratch sc = carve_sort_scratch(reinterpret_cast<WorkspaceHeader*>(temp),
                                              reinterpret_cast<char*>(temp) + kHeaderBytes, T, 4);
    const int2* r = reinterpret_cast<const int2*>(tile_ranges);
    k_tile_keys<<<grid_of(T), 256, 0, s>>>(r, T, x_blocks, morton_bucket, keys_c, tile_ids);
    if (cudaGetLastError() != cudaSuccess) return GSR_CUDA_ERROR;
    if (launch_sort32(T, nullptr, T, OrderMap{kOrderMasked, 32}, 4, keys_c, tile_ids, tile_counts, tile_order, sc,
                      s) != cudaSuccess)
        return GSR_CUDA_ERROR;
    k_tile_desc<<<grid_of(T), 256, 0, s>>>(tile_counts, tile_order, r, T, x_blocks, zigzag_group,
                                           reinterpret_cast<int4*>(tile_desc));
    return cudaGetLastError() == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
}

gsr_status gsr_tile_desc_ranges(const int32_t* tile_desc, int total_tiles, int x_blocks, int32_t* tile_ranges,
                                gsr_stream_t stream)
{
    if (total_tiles < 0 || x_blocks <= 0) return GSR_INVALID_ARG;
    if (total_tiles == 0) return GSR_OK;
    if (!tile_desc || !tile_ranges) return GSR_INVALID_ARG;
    k_desc_ranges<<<grid_of(total_tiles), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const int4*>(tile_desc), total_tiles, x_blocks, reinterpret_cast<int2*>(tile_ranges));
    return cudaGetLastError() == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
}

}  // extern "C"
