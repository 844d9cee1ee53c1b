// Tile ranges and feature gather for sm_103a.
//
// Tile ranges: the reference finds [lower_bound, upper_bound) of every tile
// by a binary search per tile (csrc/cuda_rasterizer/render.cu:10-35,
// 3510-3521) or by a boundary scan after zero-filling (render.cu:3526-3557).
// Here both results come from one coalesced pass over the sorted keys: the
// thread at boundary i (between keys i-1 and i, with virtual keys at -1 and
// M) writes start = i for every tile in (tile(i-1), tile(i)] and end = i for
// every tile in [tile(i-1), tile(i)).  That is exactly the binary-search
// answer for every tile, empty tiles included, in O(M + T) work.
#include "gsr_internal.h"

namespace gsr {
namespace {

__device__ __forceinline__ int clamp_count(int num, const int32_t* d_num, long long cap)
{
    long long n = d_num ? (long long)*d_num : (long long)num;
    if (n < 0) n = 0;
    if (n > cap) n = cap;
    return (int)n;
}

__device__ __forceinline__ uint32_t tile_of(uint64_t k) { return (uint32_t)(k >> 32); }
__device__ __forceinline__ uint32_t tile_of(uint32_t k) { return k; }

template <typename K>
__global__ void k_ranges_exact(int num, const int32_t* __restrict__ d_num, long long cap, int tiles,
                               const K* __restrict__ keys, int2* __restrict__ ranges)
{
    const int n = clamp_count(num, d_num, cap);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i <= n; i += stride) {
        int a = -1, b = tiles;  // tile(i-1), tile(i); virtual -1 and T at the ends
        if (i > 0) a = (int)min((uint32_t)tiles, tile_of(__ldg(keys + i - 1)));
        if (i < n) b = (int)min((uint32_t)tiles, tile_of(__ldg(keys + i)));
        if (a == b) continue;
        // start = i for tiles a+1 .. b (capped at T-1); end = i for tiles max(a,0) .. b-1
        const int lo = max(a, 0), hi = min(b, tiles - 1);
        for (int t = lo; t <= hi; t++) {
            if (t > a) ranges[t].x = (int)i;
            if (t < b) ranges[t].y = (int)i;
        }
    }
}

// Boundary-scan variant (empty tiles keep the zero fill).
__global__ void k_ranges_scan(int num, const int32_t* __restrict__ d_num, long long cap, int tiles,
                              const uint64_t* __restrict__ keys, int2* __restrict__ ranges)
{
    const int n = clamp_count(num, d_num, cap);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t cur = (uint32_t)(__ldg(keys + i) >> 32);
        if (cur >= (uint32_t)tiles) continue;
        if (i == 0) {
            ranges[cur].x = 0;
        } else {
            const uint32_t prev = (uint32_t)(__ldg(keys + i - 1) >> 32);
            if (cur != prev) {
                if (prev < (uint32_t)tiles) ranges[prev].y = (int)i;
                ranges[cur].x = (int)i;
            }
        }
        if (i == n - 1) ranges[cur].y = n;
    }
}

__global__ void k_zero_ranges(int tiles, int2* ranges)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < tiles; t += gridDim.x * blockDim.x)
        ranges[t] = make_int2(0, 0);
}

// dst[i] = src[values[i]] (csrc/cuda_rasterizer/gather.cu:6-22).
__global__ void k_gather(int num, const int32_t* __restrict__ d_num, long long cap,
                         const uint32_t* __restrict__ values, const float2* __restrict__ sxy,
                         const float4* __restrict__ srgbd, const float4* __restrict__ scon, float2* __restrict__ dxy,
                         float4* __restrict__ drgbd, float4* __restrict__ dcon)
{
    const int n = clamp_count(num, d_num, cap);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t g = __ldg(values + i);
        dxy[i] = __ldg(sxy + g);
        drgbd[i] = __ldg(srgbd + g);
        dcon[i] = __ldg(scon + g);
    }
}

}  // namespace

cudaError_t launch_tile_ranges(int num, const int32_t* d_num, long long cap, int tiles, const uint64_t* keys,
                               int32_t* ranges, bool scan_semantics, cudaStream_t stream)
{
    if (tiles <= 0) return cudaSuccess;
    const int sms = device_sm_count();
    int2* r = reinterpret_cast<int2*>(ranges);
    const long long work = (d_num ? cap : (long long)num) + 1;
    const int grid = (int)max(1LL, min((long long)sms * 8, (work + 255) / 256));
    if (scan_semantics) {
        k_zero_ranges<<<min(sms * 4, div_up(tiles, 256)), 256, 0, stream>>>(tiles, r);
        k_ranges_scan<<<grid, 256, 0, stream>>>(num, d_num, cap, tiles, keys, r);
    } else {
        k_ranges_exact<uint64_t><<<grid, 256, 0, stream>>>(num, d_num, cap, tiles, keys, r);
    }
    return cudaGetLastError();
}

cudaError_t launch_tile_ranges32(const int32_t* d_num, long long cap, int tiles, const uint32_t* tile_ids,
                                 int2* ranges, cudaStream_t stream)
{
    if (tiles <= 0) return cudaSuccess;
    const int sms = device_sm_count();
    const int grid = (int)max(1LL, min((long long)sms * 8, (cap + 256) / 256));
    k_ranges_exact<uint32_t><<<grid, 256, 0, stream>>>(0, d_num, cap, tiles, tile_ids, ranges);
    return cudaGetLastError();
}

cudaError_t launch_gather(int num, const int32_t* d_num, const uint32_t* values, const float2* sxy,
                          const float4* srgbd, const float4* scon, float2* dxy, float4* drgbd, float4* dcon,
                          long long cap, cudaStream_t stream)
{
    const int sms = device_sm_count();
    const long long work = d_num ? cap : (long long)num;
    if (work <= 0) return cudaSuccess;
    const int grid = (int)max(1LL, min((long long)sms * 8, (work + 255) / 256));
    k_gather<<<grid, 256, 0, stream>>>(num, d_num, cap, values, sxy, srgbd, scon, dxy, drgbd, dcon);
    return cudaGetLastError();
}

}  // namespace gsr
