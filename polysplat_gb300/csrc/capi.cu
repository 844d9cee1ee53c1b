// C ABI of the gsr library (declared in include/gsr.h).
#include <atomic>
#include <cstring>
#include <mutex>

#include "gsr_internal.h"

namespace gsr {

int current_device()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return -1;
    return dev;
}

// Failure-detection hooks: process-wide, read by every later sort launch.
static std::atomic<uint32_t> g_sort_wait_limit{kSpinLimit};
static std::atomic<int> g_sort_stall{0};

uint32_t sort_wait_limit() { return g_sort_wait_limit.load(std::memory_order_relaxed); }
bool sort_stall_first_tile() { return g_sort_stall.load(std::memory_order_relaxed) != 0; }

int device_sm_count()
{
    // one query per device; host threads may race to fill it with the same value
    static std::atomic<int> cached[kMaxDevices];
    int dev = current_device();
    if (dev < 0) dev = 0;
    int v = cached[dev].load(std::memory_order_relaxed);
    if (v == 0) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        v = n > 0 ? n : 1;
        cached[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

// Stage-timing state: `frames` rows of kMarks events; row g_prof_row is the
// one the current forward records into.
constexpr int kMarks = 16;
static cudaEvent_t* g_prof = nullptr;
static int g_prof_frames = 0;
static int g_prof_row = -1;
static int g_prof_mark = 0;
static int g_prof_marks_per_frame = 0;
static cudaError_t g_last_error = cudaSuccess;

void profile_mark(cudaStream_t stream)
{
    if (!g_prof || g_prof_row < 0 || g_prof_row >= g_prof_frames || g_prof_mark >= kMarks) return;
    cudaEventRecord(g_prof[g_prof_row * kMarks + g_prof_mark++], stream);
}

static void profile_frame_begin()
{
    if (!g_prof) return;
    if (g_prof_row >= 0 && g_prof_mark > 0) g_prof_marks_per_frame = g_prof_mark;
    g_prof_row++;
    g_prof_mark = 0;
}

static gsr_status from_cuda(cudaError_t e)
{
    if (e == cudaSuccess) return GSR_OK;
    g_last_error = e;
    if (e == cudaErrorInvalidValue) return GSR_INVALID_ARG;
    return GSR_CUDA_ERROR;
}

static int tiles_of(int W, int H, int bx, int by) { return div_up(W, bx) * div_up(H, by); }

static bool render_needs_ranges(int variant)
{
    return variant == GSR_RENDER_PERSISTENT_RANGES || variant == GSR_RENDER_RANGES_CADENCE2 ||
           variant == GSR_RENDER_DT;
}

static bool valid_tile_shape(int bx, int by)
{
    return (bx == 16 && by == 16) || (bx == 32 && by == 16) || (bx == 24 && by == 16) || (bx == 32 && by == 32);
}

gsr_status preprocess_params(PreprocessParams& p, int P, const float* pos, const void* shs,
                             const float* opacity, const float* cov3d, int width, int height, int block_x,
                             int block_y, const float* cam_pos, const float* cam_rot, float fx, float fy,
                             float zfar, float znear, float* points_xy, float* rgb_depth,
                             float* conic_opacity, uint64_t* keys, uint32_t* values, int64_t cap,
                             int32_t* curr_offset, void* workspace, size_t workspace_bytes)
{
    if (P < 0 || width <= 0 || height <= 0 || block_x <= 0 || block_y <= 0 || !cam_pos || !cam_rot || !curr_offset)
        return GSR_INVALID_ARG;
    if (P > 0 && (!pos || !shs || !opacity || !cov3d || !points_xy || !rgb_depth || !conic_opacity))
        return GSR_INVALID_ARG;
    if (cap > 0 && (!keys || !values)) return GSR_INVALID_ARG;
    p.df = DepthFirstRecords{nullptr, nullptr, nullptr, nullptr, 0};
    p.gid_base = 0;
    p.tile_base = 0;
    p.views = nullptr;
    p.n_views = 0;
    p.massive_area = kDefaultMassiveArea;
    p.huge_area = kDefaultHugeArea;
    p.quad = 0;
    p.interleave = 0;
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
    camera_matrices(width, height, cam_pos, cam_rot, fx, fy, zfar, znear, p.view, p.proj);
    p.campos[0] = cam_pos[0];
    p.campos[1] = cam_pos[1];
    p.campos[2] = cam_pos[2];
    p.tanx = width / (2.0f * fx);
    p.tany = height / (2.0f * fy);
    p.fx = fx;
    p.fy = fy;
    p.points_xy = reinterpret_cast<float2*>(points_xy);
    p.rgb_depth = reinterpret_cast<float4*>(rgb_depth);
    p.conic_opacity = reinterpret_cast<float4*>(conic_opacity);
    p.keys = keys;
    p.vals = values;
    p.cap = cap;
    p.counter = curr_offset;
    p.mq.capacity = p.mq.huge_capacity = 0;
    p.mq.entries = nullptr;
    p.mq.count = p.mq.head = p.mq.depth_hi = nullptr;
    if (workspace && workspace_bytes >= kSmallWorkspaceBytes) {
        WorkspaceHeader* h = reinterpret_cast<WorkspaceHeader*>(workspace);
        p.mq.entries = reinterpret_cast<MassiveEntry*>(reinterpret_cast<char*>(workspace) + kHeaderBytes);
        p.mq.capacity = kMassiveQueueEntries;
        p.mq.huge_capacity = kMassiveHugeEntries;
        p.mq.count = h->mq_count;
        p.mq.head = &h->mq_head[0][0];
        p.mq.depth_hi = &h->depth_hi;
    }
    return GSR_OK;
}

}  // namespace gsr

using namespace gsr;

extern "C" {

int gsr_version(void) { return 1; }

void gsr_profile_end(void)
{
    if (g_prof) {
        for (int i = 0; i < g_prof_frames * kMarks; i++)
            if (g_prof[i]) cudaEventDestroy(g_prof[i]);
        delete[] g_prof;
    }
    g_prof = nullptr;
    g_prof_frames = 0;
    g_prof_row = -1;
    g_prof_mark = 0;
    g_prof_marks_per_frame = 0;
}

gsr_status gsr_profile_begin(int frames)
{
    gsr_profile_end();
    if (frames <= 0) return GSR_INVALID_ARG;
    g_prof = new cudaEvent_t[(size_t)frames * kMarks]();
    g_prof_frames = frames;
    for (int i = 0; i < frames * kMarks; i++) {
        cudaError_t e = cudaEventCreate(&g_prof[i]);
        if (e != cudaSuccess) {
            gsr_profile_end();
            return from_cuda(e);
        }
    }
    return GSR_OK;
}

int gsr_profile_read(float* ms, int frames, int max_stages)
{
    if (!g_prof || !ms) return -1;
    if (g_prof_row >= 0 && g_prof_mark > 0) g_prof_marks_per_frame = g_prof_mark;
    const int stages = g_prof_marks_per_frame - 1;
    if (stages <= 0) return -1;
    const int rows = g_prof_row + 1 < frames ? g_prof_row + 1 : frames;
    for (int f = 0; f < rows && f < g_prof_frames; f++) {
        if (cudaEventSynchronize(g_prof[f * kMarks + stages]) != cudaSuccess) return -1;
        for (int k = 0; k < stages && k < max_stages; k++) {
            float t = 0.f;
            cudaEventElapsedTime(&t, g_prof[f * kMarks + k], g_prof[f * kMarks + k + 1]);
            ms[f * max_stages + k] = t;
        }
    }
    return stages;
}

const char* gsr_last_error(void) { return cudaGetErrorString(g_last_error); }

gsr_status gsr_debug_set_sort_wait_limit(uint32_t spins)
{
    g_sort_wait_limit.store(spins ? spins : kSpinLimit, std::memory_order_relaxed);
    return GSR_OK;
}

gsr_status gsr_debug_stall_sort(int on)
{
    g_sort_stall.store(on ? 1 : 0, std::memory_order_relaxed);
    return GSR_OK;
}

gsr_status gsr_device_check(int device)
{
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return GSR_CUDA_ERROR;
    if (prop.major != 10 || prop.minor != 3) return GSR_CUDA_ERROR;
    return GSR_OK;
}

size_t gsr_workspace_size(int64_t capacity) { return sort_workspace_bytes(capacity); }

size_t gsr_render_workspace_size(void) { return kSmallWorkspaceBytes; }

gsr_status gsr_workspace_reset(void* workspace, gsr_stream_t stream)
{
    if (!workspace) return GSR_INVALID_ARG;
    return from_cuda(cudaMemsetAsync(workspace, 0, sizeof(uint32_t), (cudaStream_t)stream));
}

gsr_status gsr_read_status(const void* workspace, const int32_t* d_num, int64_t capacity, int32_t* num_out,
                           gsr_stream_t stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaStreamSynchronize(s) != cudaSuccess) return GSR_CUDA_ERROR;
    uint32_t status = 0;
    int32_t num = 0;
    if (workspace && cudaMemcpy(&status, workspace, sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
        return GSR_CUDA_ERROR;
    if (d_num && cudaMemcpy(&num, d_num, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
        return GSR_CUDA_ERROR;
    if (num_out) *num_out = num;
    if (status & kErrTimeout) return GSR_TIMEOUT;
    if (d_num && (int64_t)num > capacity) return GSR_OVERFLOW;
    if (status & kErrOverflow) return GSR_OVERFLOW;
    if (status & kErrBadInput) return GSR_INVALID_ARG;
    return GSR_OK;
}

void gsr_camera_matrices(int width, int height, const float* cam_pos, const float* cam_rot, float focal_x,
                         float focal_y, float z_far, float z_near, float* view16, float* proj16)
{
    camera_matrices(width, height, cam_pos, cam_rot, focal_x, focal_y, z_far, z_near, view16, proj16);
}

gsr_status gsr_scene_prepare(int P, const float* log_scales, const float* quats, const float* opacity_logits,
                             float* opacity, float* cov3d, gsr_stream_t stream)
{
    if (P < 0 || (P > 0 && (!log_scales || !quats || !opacity_logits || !opacity || !cov3d))) return GSR_INVALID_ARG;
    return from_cuda(launch_scene_prepare(P, log_scales, quats, opacity_logits, opacity, cov3d, (cudaStream_t)stream));
}

static gsr_status preprocess_impl(int P, const float* pos, const void* shs, int shs_half, const float* opacity,
                                  const float* cov3d, int width, int height, int block_x, int block_y,
                                  const float* cam_pos, const float* cam_rot, float fx, float fy, float zfar,
                                  float znear, float* points_xy, float* rgb_depth, float* conic_opacity,
                                  uint64_t* keys, uint32_t* values, int64_t cap, int32_t* curr_offset,
                                  void* workspace, size_t workspace_bytes, cudaStream_t s, bool quad = false)
{
    PreprocessParams p;
    const gsr_status st = preprocess_params(p, P, pos, shs, opacity, cov3d, width, height, block_x, block_y, cam_pos,
                                            cam_rot, fx, fy, zfar, znear, points_xy, rgb_depth, conic_opacity, keys,
                                            values, cap, curr_offset, workspace, workspace_bytes);
    if (st != GSR_OK) return st;
    p.quad = quad ? 1 : 0;
    return from_cuda(launch_preprocess(p, shs_half != 0, s));
}

gsr_status gsr_preprocess(int P, const float* pos, const void* shs, int shs_half, const float* opacity,
                          const float* cov3d, int width, int height, int block_x, int block_y, const float* cam_pos,
                          const float* cam_rot, float focal_x, float focal_y, float z_far, float z_near,
                          float* points_xy, float* rgb_depth, float* conic_opacity, uint64_t* keys, uint32_t* values,
                          int64_t key_capacity, int32_t* curr_offset, void* workspace, size_t workspace_bytes,
                          gsr_stream_t stream)
{
    return preprocess_impl(P, pos, shs, shs_half, opacity, cov3d, width, height, block_x, block_y, cam_pos, cam_rot,
                           focal_x, focal_y, z_far, z_near, points_xy, rgb_depth, conic_opacity, keys, values,
                           key_capacity, curr_offset, workspace, workspace_bytes, (cudaStream_t)stream);
}

static gsr_status sort_impl(int num, const int32_t* d_num, int end_bit, void* workspace, size_t workspace_bytes,
                            const uint64_t* keys_in, const uint32_t* values_in, uint64_t* keys_out,
                            uint32_t* values_out, int64_t capacity, bool compress_depth, cudaStream_t stream)
{
    if (!workspace || end_bit < 1 || end_bit > 64 || capacity < 0 || (!d_num && num < 0)) return GSR_INVALID_ARG;
    if (!d_num && num > capacity) return GSR_INVALID_ARG;
    if (capacity > 0 && (!keys_in || !values_in || !keys_out || !values_out)) return GSR_INVALID_ARG;
    if (keys_in == keys_out || values_in == values_out) return GSR_INVALID_ARG;
    SortArgs a;
    a.num = num;
    a.d_num = d_num;
    a.cap = capacity;
    a.end_bit = end_bit;
    a.keys_in = keys_in;
    a.vals_in = values_in;
    a.keys_out = keys_out;
    a.vals_out = values_out;
    a.ws = workspace;
    a.ws_bytes = workspace_bytes;
    a.compress_depth = compress_depth;
    return from_cuda(launch_sort(a, stream));
}

gsr_status gsr_sort_bits(int num, const int32_t* d_num, int end_bit, void* workspace, size_t workspace_bytes,
                         const uint64_t* keys_in, const uint32_t* values_in, uint64_t* keys_out, uint32_t* values_out,
                         int64_t capacity, gsr_stream_t stream)
{
    return sort_impl(num, d_num, end_bit, workspace, workspace_bytes, keys_in, values_in, keys_out, values_out,
                     capacity, false, (cudaStream_t)stream);
}

gsr_status gsr_sort(int num, const int32_t* d_num, int width, int height, int block_x, int block_y, void* workspace,
                    size_t workspace_bytes, const uint64_t* keys_in, const uint32_t* values_in, uint64_t* keys_out,
                    uint32_t* values_out, int64_t capacity, gsr_stream_t stream)
{
    if (width <= 0 || height <= 0 || block_x <= 0 || block_y <= 0) return GSR_INVALID_ARG;
    const int end_bit = 32 + bits_for((uint32_t)tiles_of(width, height, block_x, block_y));
    return gsr_sort_bits(num, d_num, end_bit, workspace, workspace_bytes, keys_in, values_in, keys_out, values_out,
                         capacity, stream);
}

gsr_status gsr_tile_ranges(int num, const int32_t* d_num, int width, int height, int block_x, int block_y,
                           const uint64_t* keys_sorted, int32_t* ranges, int scan_semantics, gsr_stream_t stream)
{
    if (width <= 0 || height <= 0 || block_x <= 0 || block_y <= 0 || !ranges || (!d_num && num < 0))
        return GSR_INVALID_ARG;
    const long long cap = d_num ? (long long)INT32_MAX : (long long)num;
    return from_cuda(launch_tile_ranges(num, d_num, cap, tiles_of(width, height, block_x, block_y), keys_sorted,
                                        ranges, scan_semantics != 0, (cudaStream_t)stream));
}

gsr_status gsr_gather(int num, const int32_t* d_num, const uint32_t* values, const float* src_xy,
                      const float* src_rgb_depth, const float* src_conic, float* dst_xy, float* dst_rgb_depth,
                      float* dst_conic, gsr_stream_t stream)
{
    if (!d_num && num < 0) return GSR_INVALID_ARG;
    if (d_num) return GSR_INVALID_ARG;  // the destination size must be known: pass the host count
    return from_cuda(launch_gather(num, nullptr, values, reinterpret_cast<const float2*>(src_xy),
                                   reinterpret_cast<const float4*>(src_rgb_depth),
                                   reinterpret_cast<const float4*>(src_conic), reinterpret_cast<float2*>(dst_xy),
                                   reinterpret_cast<float4*>(dst_rgb_depth), reinterpret_cast<float4*>(dst_conic),
                                   (long long)num, (cudaStream_t)stream));
}

static gsr_status render_impl(int variant, int num, const int32_t* d_num, long long cap, int width, int height,
                              int block_x, int block_y, int P, const float* points_xy, const float* rgb_depth,
                              const float* conic_opacity, const uint64_t* keys_sorted, const uint32_t* values_sorted,
                              const int32_t* ranges, const float* bg_color, uint8_t* out_color, void* workspace,
                              cudaStream_t s, bool quad = false)
{
    if (!workspace || !out_color || !bg_color || width <= 0 || height <= 0 || !valid_tile_shape(block_x, block_y))
        return GSR_INVALID_ARG;
    if (quad && (block_x != 16 || block_y != 16 || variant == GSR_RENDER_SPLIT)) return GSR_INVALID_ARG;
    if (render_needs_ranges(variant) ? !ranges : (!keys_sorted && !ranges)) return GSR_INVALID_ARG;
    if (variant < 0 || variant > GSR_RENDER_SPLIT) return GSR_INVALID_ARG;
    RenderArgs a;
    a.variant = variant;
    a.num = num;
    a.d_num = d_num;
    a.cap = cap;
    a.W = width;
    a.H = height;
    a.bx = block_x;
    a.by = block_y;
    a.P = P;
    a.xy = reinterpret_cast<const float2*>(points_xy);
    a.rgbd = reinterpret_cast<const float4*>(rgb_depth);
    a.con = reinterpret_cast<const float4*>(conic_opacity);
    a.keys = keys_sorted;
    a.vals = values_sorted;
    a.ranges = reinterpret_cast<const int2*>(ranges);
    a.bg[0] = bg_color[0];
    a.bg[1] = bg_color[1];
    a.bg[2] = bg_color[2];
    a.out = out_color;
    a.ws = reinterpret_cast<WorkspaceHeader*>(workspace);
    a.quad = quad ? 1 : 0;
    return from_cuda(launch_render(a, s));
}

gsr_status gsr_render(int variant, int num, const int32_t* d_num, int width, int height, int block_x, int block_y,
                      int P, const float* points_xy, const float* rgb_depth, const float* conic_opacity,
                      const uint64_t* keys_sorted, const uint32_t* values_sorted, const int32_t* ranges,
                      const float* bg_color, uint8_t* out_color, void* workspace, gsr_stream_t stream)
{
    if (!d_num && num < 0) return GSR_INVALID_ARG;
    return render_impl(variant, num, d_num, d_num ? (long long)INT32_MAX : (long long)num, width, height, block_x,
                       block_y, P, points_xy, rgb_depth, conic_opacity, keys_sorted, values_sorted, ranges, bg_color,
                       out_color, workspace, (cudaStream_t)stream);
}

gsr_status gsr_forward(int variant, int P, const float* pos, const void* shs, int shs_half, const float* opacity,
                       const float* cov3d, int width, int height, int block_x, int block_y, const float* cam_pos,
                       const float* cam_rot, float focal_x, float focal_y, float z_far, float z_near,
                       int32_t* curr_offset, void* workspace, size_t workspace_bytes, uint64_t* keys_unsorted,
                       uint32_t* values_unsorted, uint64_t* keys_sorted, uint32_t* values_sorted,
                       int64_t key_capacity, float* points_xy, float* rgb_depth, float* conic_opacity,
                       int32_t* ranges, const float* bg_color, uint8_t* out_color, gsr_stream_t stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    // GSR_QUAD_KEYS: one key per 2x2 group of 16x16 tiles, same image
    const bool quad = (variant & GSR_QUAD_KEYS) != 0;
    variant &= ~GSR_QUAD_KEYS;
    if (!workspace || !curr_offset || !valid_tile_shape(block_x, block_y)) return GSR_INVALID_ARG;
    if (quad && (block_x != 16 || block_y != 16 || variant == GSR_RENDER_SPLIT || P > (int)kQuadGidMask))
        return GSR_INVALID_ARG;
    if (render_needs_ranges(variant) && !ranges) return GSR_INVALID_ARG;
    if (workspace_bytes < sort_workspace_bytes(key_capacity)) return GSR_INVALID_ARG;
    profile_frame_begin();
    cudaError_t e = cudaMemsetAsync(workspace, 0, sizeof(uint32_t), s);  // status word
    if (e == cudaSuccess) e = cudaMemsetAsync(curr_offset, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return from_cuda(e);
    profile_mark(s);
    gsr_status st = preprocess_impl(P, pos, shs, shs_half, opacity, cov3d, width, height, block_x, block_y, cam_pos,
                                    cam_rot, focal_x, focal_y, z_far, z_near, points_xy, rgb_depth, conic_opacity,
                                    keys_unsorted, values_unsorted, key_capacity, curr_offset, workspace,
                                    workspace_bytes, s, quad);
    if (st != GSR_OK) return st;
    profile_mark(s);
    // key tile ids: tiles, or quads
    const int tiles = quad ? quad_cols(div_up(width, 16)) * quad_cols(div_up(height, 16))
                           : tiles_of(width, height, block_x, block_y);
    // the preprocess recorded the depth range in the workspace header: sort
    // the (tile, depth - floor) word in as few passes as it needs
    st = sort_impl(0, curr_offset, 32 + bits_for((uint32_t)tiles), workspace, workspace_bytes, keys_unsorted,
                   values_unsorted, keys_sorted, values_sorted, key_capacity, true, s);
    if (st != GSR_OK) return st;
    // tile ranges by one O(M + T) pass: the caller's buffer, else the
    // workspace's range area (too many tiles for it: the render searches)
    if (!ranges && tiles <= kWorkspaceRangeTiles) ranges = reinterpret_cast<int32_t*>(workspace_ranges(workspace, key_capacity));
    if (ranges) {
        e = launch_tile_ranges(0, curr_offset, key_capacity, tiles, keys_sorted, ranges, false, s);
        if (e != cudaSuccess) return from_cuda(e);
        profile_mark(s);
    }
    st = render_impl(variant, 0, curr_offset, key_capacity, width, height, block_x, block_y, P, points_xy, rgb_depth,
                     conic_opacity, keys_sorted, values_sorted, ranges, bg_color, out_color, workspace, s, quad);
    if (st == GSR_OK) profile_mark(s);
    return st;
}

size_t gsr_depth_first_scratch_size(int P) { return P < 0 ? 0 : df_scratch_bytes(P); }

gsr_status gsr_forward_depth_first(int variant, int P, const float* pos, const void* shs, int shs_half,
                                   const float* opacity, const float* cov3d, int width, int height, int block_x,
                                   int block_y, const float* cam_pos, const float* cam_rot, float focal_x,
                                   float focal_y, float z_far, float z_near, int32_t* curr_offset, void* workspace,
                                   size_t workspace_bytes, void* scene_scratch, size_t scene_scratch_bytes,
                                   uint32_t* tiles_unsorted, uint32_t* values_unsorted, uint32_t* tiles_sorted,
                                   uint32_t* values_sorted, int64_t key_capacity, float* points_xy, float* rgb_depth,
                                   float* conic_opacity, int32_t* ranges, const float* bg_color, uint8_t* out_color,
                                   gsr_stream_t stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    // GSR_QUAD_KEYS: the pairs name 2x2 groups of 16x16 tiles, same image
    const bool quad = (variant & GSR_QUAD_KEYS) != 0;
    variant &= ~GSR_QUAD_KEYS;
    if (!workspace || !curr_offset || !scene_scratch || !valid_tile_shape(block_x, block_y)) return GSR_INVALID_ARG;
    if (variant < 0 || variant > GSR_RENDER_SPLIT) return GSR_INVALID_ARG;
    if (quad && (block_x != 16 || block_y != 16 || variant == GSR_RENDER_SPLIT || P > (int)kQuadGidMask))
        return GSR_INVALID_ARG;
    if (workspace_bytes < sort_workspace_bytes(key_capacity) || key_capacity >= (1LL << 30)) return GSR_INVALID_ARG;
    if (P < 0 || scene_scratch_bytes < df_scratch_bytes(P)) return GSR_INVALID_ARG;
    if (key_capacity > 0 && (!tiles_unsorted || !values_unsorted || !tiles_sorted || !values_sorted))
        return GSR_INVALID_ARG;
    if (tiles_unsorted == tiles_sorted || values_unsorted == values_sorted) return GSR_INVALID_ARG;
    // pair tile ids: tiles, or quads
    const int tiles = quad ? quad_cols(div_up(width, 16)) * quad_cols(div_up(height, 16))
                           : tiles_of(width, height, block_x, block_y);
    if (!ranges) {
        if (tiles > kWorkspaceRangeTiles) return GSR_INVALID_ARG;
        ranges = reinterpret_cast<int32_t*>(workspace_ranges(workspace, key_capacity));
    }
    PreprocessParams p;
    // the counting pass emits no 64-bit keys: the key pointers only pass the checks
    gsr_status st = preprocess_params(p, P, pos, shs, opacity, cov3d, width, height, block_x, block_y, cam_pos, cam_rot,
                                      focal_x, focal_y, z_far, z_near, points_xy, rgb_depth, conic_opacity,
                                      reinterpret_cast<uint64_t*>(tiles_unsorted), values_unsorted, key_capacity,
                                      curr_offset, workspace, workspace_bytes);
    if (st != GSR_OK) return st;
    p.quad = quad ? 1 : 0;
    profile_frame_begin();
    cudaError_t e = cudaMemsetAsync(workspace, 0, sizeof(uint32_t), s);  // status word
    if (e == cudaSuccess) e = cudaMemsetAsync(curr_offset, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return from_cuda(e);
    profile_mark(s);
    e = launch_depth_first(p, shs_half != 0, scene_scratch, scene_scratch_bytes,
                           reinterpret_cast<WorkspaceHeader*>(workspace), workspace_sort_scratch(workspace, key_capacity),
                           tiles, tiles_unsorted, values_unsorted, tiles_sorted, values_sorted,
                           reinterpret_cast<int2*>(ranges), s);
    if (e != cudaSuccess) return from_cuda(e);
    st = render_impl(variant, 0, curr_offset, key_capacity, width, height, block_x, block_y, P, points_xy, rgb_depth,
                     conic_opacity, nullptr, values_sorted, ranges, bg_color, out_color, workspace, s, quad);
    if (st == GSR_OK) profile_mark(s);
    return st;
}

}  // extern "C"
