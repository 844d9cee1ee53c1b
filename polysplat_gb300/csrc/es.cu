// The reference's ES ("early sorting") helper operators (csrc/pybind.cpp:
// 183-330; preprocess.cu:673-1248; sort.cu:151-285) on this library's
// kernels, with the reference's buffer layouts:
//   pass A            counting preprocess into tiles_per_gauss [P] i32,
//                     conic_power_raw [P,4] (raw conic, power),
//                     depth_natural [P] (FLT_MAX when culled) and
//                     rect_bounds [P,2] (x | y << 16 of rect_min, rect_max);
//   depth sort + scan perm = Gaussians by depth (stable), counts gathered in
//                     that order, exclusive scan, total as a device scalar;
//   pass B            (tile id, index) pairs in depth order at the offsets;
//   tile sort         stable sort of the 32-bit tile ids over their bit width,
//                     plus the 64-bit keys tile << 32 the range search reads.
// The library's own depth-first forward (gsr_forward_depth_first) does the
// same in one call; these are the reference's separate steps.
#include <algorithm>
#include <climits>
#include <cstring>

#include "gsr_internal.h"

namespace gsr {
namespace {

constexpr int kEsScanTile = 2048;

__global__ void k_iota(int P, uint32_t* out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) out[i] = (uint32_t)i;
}

__global__ void k_gather_counts(int P, const uint32_t* __restrict__ perm, const int32_t* __restrict__ counts,
                                int32_t* __restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        const uint32_t g = perm[i];
        out[i] = g < (uint32_t)P ? counts[g] : 0;
    }
}

// exclusive scan of P int32 counts: tile sums, one-block scan of the sums,
// then each tile's scan with its offset
__global__ __launch_bounds__(256) void k_tile_sums(int P, const int32_t* __restrict__ in, uint32_t* __restrict__ sums)
{
    __shared__ uint32_t s_w[8];
    const long long base = (long long)blockIdx.x * kEsScanTile;
    uint32_t v = 0;
    for (int k = 0; k < kEsScanTile / 256; k++) {
        const long long i = base + threadIdx.x + 256 * k;
        if (i < P) v += (uint32_t)max(0, in[i]);
    }
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(GSR_FULL_MASK, v, d);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < 8; w++) t += s_w[w];
        sums[blockIdx.x] = t;
    }
}

__global__ __launch_bounds__(1024) void k_scan_sums(int nb, uint32_t* __restrict__ sums, int32_t* __restrict__ total)
{
    __shared__ uint32_t s_w[32];
    const int per = (nb + 1023) / 1024, j0 = threadIdx.x * per;
    uint32_t v = 0;
    for (int j = j0; j < min(nb, j0 + per); j++) v += sums[j];
    uint32_t incl = v;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t n = __shfl_up_sync(GSR_FULL_MASK, incl, d);
        if (lane >= (unsigned)d) incl += n;
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
    if (threadIdx.x == 0) *total = (int32_t)all;
}

__global__ __launch_bounds__(256) void k_tile_scan(int P, const int32_t* __restrict__ in,
                                                   const uint32_t* __restrict__ sums, int32_t* __restrict__ out)
{
    __shared__ uint32_t s_w[8];
    const long long base = (long long)blockIdx.x * kEsScanTile + threadIdx.x * (kEsScanTile / 256);
    uint32_t c[kEsScanTile / 256], v = 0;
    for (int k = 0; k < kEsScanTile / 256; k++) {
        const long long i = base + k;
        c[k] = i < P ? (uint32_t)max(0, in[i]) : 0u;
        v += c[k];
    }
    uint32_t incl = v;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t n = __shfl_up_sync(GSR_FULL_MASK, incl, d);
        if (lane >= (unsigned)d) incl += n;
    }
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    uint32_t wpre = 0;
    for (int w = 0; w < 8; w++)
        if (w < (int)warp) wpre += s_w[w];
    uint32_t run = sums[blockIdx.x] + wpre + incl - v;
    for (int k = 0; k < kEsScanTile / 256; k++) {
        const long long i = base + k;
        if (i < P) out[i] = (int32_t)run;
        run += c[k];
    }
}

__global__ void k_rebuild_keys(int num, const uint32_t* __restrict__ tiles, uint64_t* __restrict__ keys)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num; i += gridDim.x * blockDim.x)
        keys[i] = (uint64_t)tiles[i] << 32;
}

int grid_for(long long n) { return (int)std::max(1LL, std::min((long long)device_sm_count() * 8, (n + 255) / 256)); }

// sort scratch carved from a caller buffer: header, then the radix-sort scratch
bool carve(void* space, size_t bytes, long long cap, SortScratch& s)
{
    if (!space || bytes < kHeaderBytes + sort_scratch_bytes(cap, 4)) return false;
    s = carve_sort_scratch(reinterpret_cast<WorkspaceHeader*>(space), reinterpret_cast<char*>(space) + kHeaderBytes,
                           cap, 4);
    return true;
}

}  // namespace
}  // namespace gsr

using namespace gsr;

extern "C" {

gsr_status gsr_es_pass_a(int P, const float* pos, const void* shs, int shs_half, const float* opacity,
                         const float* cov3d, int width, int height, int block_x, int block_y, const float* cam_pos,
                         const float* cam_rot, float focal_x, float focal_y, float z_far, float z_near,
                         float* points_xy, float* rgb_depth, float* conic_opacity, int32_t* tiles_per_gauss,
                         float* conic_power_raw, float* depth_natural, int32_t* rect_bounds, gsr_stream_t stream)
{
    if (P < 0 || width <= 0 || height <= 0 || block_x <= 0 || block_y <= 0 || !cam_pos || !cam_rot) return GSR_INVALID_ARG;
    if (P > 0 && (!pos || !shs || !opacity || !cov3d || !points_xy || !rgb_depth || !conic_opacity || !tiles_per_gauss ||
                  !conic_power_raw || !depth_natural || !rect_bounds))
        return GSR_INVALID_ARG;
    PreprocessParams p;
    std::memset(&p, 0, sizeof(p));
    p.P = P;
    p.pos = pos;
    p.shs = shs;
    p.opacity = opacity;
    p.cov3d = cov3d;
    p.W = width;
    p.H = height;
    p.bx = block_x;
    p.by = block_y;
    p.gx = div_up(width, block_x);
    p.gy = div_up(height, block_y);
    camera_matrices(width, height, cam_pos, cam_rot, focal_x, focal_y, z_far, z_near, p.view, p.proj);
    for (int k = 0; k < 3; k++) p.campos[k] = cam_pos[k];
    p.tanx = width / (2.0f * focal_x);
    p.tany = height / (2.0f * focal_y);
    p.fx = focal_x;
    p.fy = focal_y;
    p.points_xy = reinterpret_cast<float2*>(points_xy);
    p.rgb_depth = reinterpret_cast<float4*>(rgb_depth);
    p.conic_opacity = reinterpret_cast<float4*>(conic_opacity);
    // no large-Gaussian queue (the thresholds exceed every area): every count
    // is made by the Gaussian's own warp, and no queue counter is touched
    p.massive_area = INT_MAX;
    p.huge_area = INT_MAX;
    p.df.count = reinterpret_cast<uint32_t*>(tiles_per_gauss);
    p.df.dkey = reinterpret_cast<uint32_t*>(depth_natural);
    p.df.geo = reinterpret_cast<float4*>(conic_power_raw);
    p.df.rect = reinterpret_cast<int2*>(rect_bounds);
    p.df.ref_layout = 1;
    const cudaError_t e = launch_preprocess_count(p, shs_half != 0, (cudaStream_t)stream);
    return e == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
}

size_t gsr_es_scan_buffer_size(int P) { return P < 0 ? 0 : (size_t)4 * ((size_t)P / kEsScanTile + 1) + 256; }

gsr_status gsr_es_depth_sort_and_scan(int P, const int32_t* tiles_per_gauss, const float* depth_natural,
                                      uint32_t* identity, uint32_t* perm, float* depth_sorted,
                                      int32_t* tiles_per_gauss_sorted, int32_t* cum_offsets_sorted,
                                      int32_t* total_out, void* sort_space, size_t sort_bytes, void* scan_space,
                                      size_t scan_bytes, gsr_stream_t stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (P < 0 || !total_out) return GSR_INVALID_ARG;
    if (P == 0) return cudaMemsetAsync(total_out, 0, sizeof(int32_t), s) == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
    if (!tiles_per_gauss || !depth_natural || !identity || !perm || !depth_sorted || !tiles_per_gauss_sorted ||
        !cum_offsets_sorted || !scan_space || scan_bytes < gsr_es_scan_buffer_size(P) || P >= (1 << 30))
        return GSR_INVALID_ARG;
    SortScratch sc;
    if (!carve(sort_space, sort_bytes, P, sc)) return GSR_INVALID_ARG;
    k_iota<<<grid_for(P), 256, 0, s>>>(P, identity);
    // positive float depths order as their bit patterns; FLT_MAX (culled) last
    const OrderMap order{kOrderMasked, 32};
    cudaError_t e = launch_sort32(P, nullptr, P, order, 4, reinterpret_cast<const uint32_t*>(depth_natural), identity,
                                  reinterpret_cast<uint32_t*>(depth_sorted), perm, sc, s);
    if (e != cudaSuccess) return GSR_CUDA_ERROR;
    k_gather_counts<<<grid_for(P), 256, 0, s>>>(P, perm, tiles_per_gauss, tiles_per_gauss_sorted);
    const int nb = div_up(P, kEsScanTile);
    uint32_t* sums = reinterpret_cast<uint32_t*>(scan_space);
    k_tile_sums<<<nb, 256, 0, s>>>(P, tiles_per_gauss_sorted, sums);
    k_scan_sums<<<1, 1024, 0, s>>>(nb, sums, total_out);
    k_tile_scan<<<nb, 256, 0, s>>>(P, tiles_per_gauss_sorted, sums, cum_offsets_sorted);
    return cudaGetLastError() == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
}

gsr_status gsr_es_pass_b(int P, int width, int height, int block_x, int block_y, const uint32_t* perm,
                         const int32_t* cum_offsets_sorted, const int32_t* tiles_per_gauss_sorted,
                         const float* points_xy, const float* conic_power_raw, const int32_t* rect_bounds,
                         uint32_t* tile_keys_unsorted, uint32_t* values_unsorted, int64_t capacity,
                         gsr_stream_t stream)
{
    if (P < 0 || width <= 0 || height <= 0 || block_x <= 0 || block_y <= 0 || capacity < 0) return GSR_INVALID_ARG;
    if (P > 0 && (!perm || !cum_offsets_sorted || !tiles_per_gauss_sorted || !points_xy || !conic_power_raw ||
                  !rect_bounds || (capacity > 0 && (!tile_keys_unsorted || !values_unsorted))))
        return GSR_INVALID_ARG;
    const cudaError_t e = launch_es_pass_b(
        P, block_x, block_y, div_up(width, block_x), perm, cum_offsets_sorted, tiles_per_gauss_sorted,
        reinterpret_cast<const float2*>(points_xy), reinterpret_cast<const float4*>(conic_power_raw),
        reinterpret_cast<const int2*>(rect_bounds), tile_keys_unsorted, values_unsorted, capacity,
        (cudaStream_t)stream);
    return e == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
}

gsr_status gsr_es_tile_sort(int num, int width, int height, int block_x, int block_y, const uint32_t* tile_keys_unsorted,
                            const uint32_t* values_unsorted, uint32_t* tile_keys_sorted, uint32_t* values_sorted,
                            uint64_t* keys_sorted_out, void* sort_space, size_t sort_bytes, gsr_stream_t stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (num < 0 || width <= 0 || height <= 0 || block_x <= 0 || block_y <= 0) return GSR_INVALID_ARG;
    if (num == 0) return GSR_OK;
    if (!tile_keys_unsorted || !values_unsorted || !tile_keys_sorted || !values_sorted || !keys_sorted_out ||
        num >= (1 << 30))
        return GSR_INVALID_ARG;
    SortScratch sc;
    if (!carve(sort_space, sort_bytes, num, sc)) return GSR_INVALID_ARG;
    const int bits = bits_for((uint32_t)(div_up(width, block_x) * div_up(height, block_y)));
    const OrderMap order{kOrderMasked, bits, 0};  // tile ids
    cudaError_t e = launch_sort32(num, nullptr, num, order, (bits + 7) / 8, tile_keys_unsorted, values_unsorted,
                                  tile_keys_sorted, values_sorted, sc, s);
    if (e != cudaSuccess) return GSR_CUDA_ERROR;
    k_rebuild_keys<<<grid_for(num), 256, 0, s>>>(num, tile_keys_sorted, keys_sorted_out);
    return cudaGetLastError() == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
}

}  // extern "C"
