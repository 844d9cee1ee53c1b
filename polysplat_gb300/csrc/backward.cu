// Differentiable forward and backward of the rasterizer (no counterpart in
// the reference, which renders only): the C ABI entries and the preprocess
// adjoint kernel.  The per-Gaussian adjoint is adjoint.h (checked in double
// against central differences); the render backward is in render.cu.
#include <algorithm>
#include <vector>

#include "adjoint.h"
#include "gsr_internal.h"

namespace gsr {
namespace {

struct PreBackArgs {
    int P;
    const float* means;
    const float* log_scales;
    const float* quats;
    const float* logits;
    const float* shs;  // [P,48] f32
    gsr_adj::Cam<float> cam;
    const float* gxy;
    const float* gcon;
    const float* grgb;
    float* g_means;
    float* g_log_scales;
    float* g_quats;
    float* g_logits;
    float* g_shs;
    int accumulate;
};

// One thread per Gaussian: recompute the forward, apply the adjoint.
// Gaussians that reached no pixel carry zero gradients and are skipped
// (written as zeros unless accumulating).
__global__ __launch_bounds__(128) void k_preprocess_backward(const __grid_constant__ PreBackArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.P) return;
    float gxy[2] = {a.gxy[2 * (size_t)i], a.gxy[2 * (size_t)i + 1]};
    float gcon[4], grgb[3];
    bool any = gxy[0] != 0.f || gxy[1] != 0.f;
    for (int k = 0; k < 4; k++) {
        gcon[k] = a.gcon[4 * (size_t)i + k];
        any |= gcon[k] != 0.f;
    }
    for (int k = 0; k < 3; k++) {
        grgb[k] = a.grgb[3 * (size_t)i + k];
        any |= grgb[k] != 0.f;
    }
    float gm[3] = {0.f, 0.f, 0.f}, gls[3] = {0.f, 0.f, 0.f}, gq[4] = {0.f, 0.f, 0.f, 0.f}, glogit = 0.f;
    float gsh[48];
    for (int k = 0; k < 48; k++) gsh[k] = 0.f;
    if (any) {
        float m[3], ls[3], q[4], sh[48];
        for (int k = 0; k < 3; k++) {
            m[k] = a.means[3 * (size_t)i + k];
            ls[k] = a.log_scales[3 * (size_t)i + k];
        }
        for (int k = 0; k < 4; k++) q[k] = a.quats[4 * (size_t)i + k];
        for (int k = 0; k < 48; k++) sh[k] = a.shs[48 * (size_t)i + k];
        gsr_adj::Fwd<float> f;
        gsr_adj::Tape<float> tp;
        gsr_adj::forward(m, ls, q, a.logits[i], sh, a.cam, f, tp);
        gsr_adj::backward(m, sh, a.cam, tp, gxy, gcon, grgb, gm, gls, gq, glogit, gsh);
    } else if (a.accumulate) {
        return;
    }
    auto put = [&](float* dst, size_t off, float v) { dst[off] = a.accumulate ? dst[off] + v : v; };
    for (int k = 0; k < 3; k++) {
        put(a.g_means, 3 * (size_t)i + k, gm[k]);
        put(a.g_log_scales, 3 * (size_t)i + k, gls[k]);
    }
    for (int k = 0; k < 4; k++) put(a.g_quats, 4 * (size_t)i + k, gq[k]);
    put(a.g_logits, i, glogit);
    for (int k = 0; k < 48; k++) put(a.g_shs, 48 * (size_t)i + k, gsh[k]);
}

// Views of one multi-view adjoint launch (more views take several launches,
// the later ones accumulating).
constexpr int kAdjViews = 16;

struct PreBackViewsArgs {
    int P, n_views;
    const float* means;
    const float* log_scales;
    const float* quats;
    const float* logits;
    const float* shs;  // [P,48] f32
    gsr_adj::Cam<float> cam[kAdjViews];
    // per-view gradient records of the screen-space features (conic and
    // opacity, xy, colour; 12 floats): view v's rows start at v * P (of the
    // launch's first view)
    const float4* grec;
    float* g_means;
    float* g_log_scales;
    float* g_quats;
    float* g_logits;
    float* g_shs;
    int accumulate;
};

// One thread per Gaussian over all views of the launch: the parameters are
// read once, each view that saw the Gaussian replays its forward and adds
// its adjoint, and the sums are written once.
__global__ __launch_bounds__(128) void k_preprocess_backward_views(const __grid_constant__ PreBackViewsArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.P) return;
    float gm[3] = {0.f, 0.f, 0.f}, gls[3] = {0.f, 0.f, 0.f}, gq[4] = {0.f, 0.f, 0.f, 0.f}, glogit = 0.f;
    float gsh[48];
    for (int k = 0; k < 48; k++) gsh[k] = 0.f;
    float m[3], ls[3], q[4], sh[48], logit = 0.f;
    bool loaded = false;
    for (int v = 0; v < a.n_views; v++) {
        const size_t r = (size_t)v * a.P + i;
        const float4 q0 = a.grec[3 * r], q1 = a.grec[3 * r + 1], q2 = a.grec[3 * r + 2];
        float gcon[4] = {q0.x, q0.y, q0.z, q0.w}, gxy[2] = {q1.x, q1.y}, grgb[3] = {q1.z, q1.w, q2.x};
        const bool any = gcon[0] != 0.f || gcon[1] != 0.f || gcon[2] != 0.f || gcon[3] != 0.f || gxy[0] != 0.f ||
                         gxy[1] != 0.f || grgb[0] != 0.f || grgb[1] != 0.f || grgb[2] != 0.f;
        if (!any) continue;
        if (!loaded) {
            for (int k = 0; k < 3; k++) {
                m[k] = a.means[3 * (size_t)i + k];
                ls[k] = a.log_scales[3 * (size_t)i + k];
            }
            for (int k = 0; k < 4; k++) q[k] = a.quats[4 * (size_t)i + k];
            for (int k = 0; k < 48; k++) sh[k] = a.shs[48 * (size_t)i + k];
            logit = a.logits[i];
            loaded = true;
        }
        gsr_adj::Fwd<float> f;
        gsr_adj::Tape<float> tp;
        gsr_adj::forward(m, ls, q, logit, sh, a.cam[v], f, tp);
        float vm[3], vls[3], vq[4], vlogit;
        gsr_adj::backward<float, true>(m, sh, a.cam[v], tp, gxy, gcon, grgb, vm, vls, vq, vlogit, gsh);
        for (int k = 0; k < 3; k++) {
            gm[k] += vm[k];
            gls[k] += vls[k];
        }
        for (int k = 0; k < 4; k++) gq[k] += vq[k];
        glogit += vlogit;
    }
    if (!loaded && a.accumulate) return;
    auto put = [&](float* dst, size_t off, float v) { dst[off] = a.accumulate ? dst[off] + v : v; };
    for (int k = 0; k < 3; k++) {
        put(a.g_means, 3 * (size_t)i + k, gm[k]);
        put(a.g_log_scales, 3 * (size_t)i + k, gls[k]);
    }
    for (int k = 0; k < 4; k++) put(a.g_quats, 4 * (size_t)i + k, gq[k]);
    put(a.g_logits, i, glogit);
    for (int k = 0; k < 48; k++) put(a.g_shs, 48 * (size_t)i + k, gsh[k]);
}

gsr_adj::Cam<float> adj_camera(int W, int H, const float* cam_pos, const float* cam_rot, float fx, float fy,
                               float zfar, float znear)
{
    gsr_adj::Cam<float> c;
    camera_matrices(W, H, cam_pos, cam_rot, fx, fy, zfar, znear, c.view, c.proj);
    for (int k = 0; k < 3; k++) c.campos[k] = cam_pos[k];
    c.fx = fx;
    c.fy = fy;
    c.tanx = W / (2.0f * fx);
    c.tany = H / (2.0f * fy);
    c.W = W;
    c.H = H;
    return c;
}

}  // namespace
}  // namespace gsr

using namespace gsr;

extern "C" {

gsr_status gsr_train_forward(int P, const float* means, const float* log_scales, const float* quats,
                             const float* logits, const float* shs, int width, int height, const float* cam_pos,
                             const float* cam_rot, float focal_x, float focal_y, float z_far, float z_near,
                             const float* bg_color, float* opacity, float* cov3d, int32_t* curr_offset,
                             void* workspace, size_t workspace_bytes, uint64_t* keys_unsorted,
                             uint32_t* values_unsorted, uint64_t* keys_sorted, uint32_t* values_sorted,
                             int64_t key_capacity, float* points_xy, float* rgb_depth, float* conic_opacity,
                             int32_t* ranges, int32_t* n_tile, float* T_final, float* image, gsr_stream_t stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (P < 0 || width <= 0 || height <= 0 || !cam_pos || !cam_rot || !bg_color || !curr_offset || !workspace ||
        !ranges || !n_tile || !T_final || !image || !opacity || !cov3d)
        return GSR_INVALID_ARG;
    if (P > 0 && (!means || !log_scales || !quats || !logits || !shs)) return GSR_INVALID_ARG;
    if (workspace_bytes < sort_workspace_bytes(key_capacity) || key_capacity >= (1LL << 30)) return GSR_INVALID_ARG;
    const int tiles = div_up(width, 16) * div_up(height, 16);
    cudaError_t e = launch_scene_prepare(P, log_scales, quats, logits, opacity, cov3d, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(workspace, 0, sizeof(uint32_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(curr_offset, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return GSR_CUDA_ERROR;
    gsr_status st = gsr_preprocess(P, means, shs, 0, opacity, cov3d, width, height, 16, 16, cam_pos, cam_rot,
                                   focal_x, focal_y, z_far, z_near, points_xy, rgb_depth, conic_opacity,
                                   keys_unsorted, values_unsorted, key_capacity, curr_offset, workspace,
                                   workspace_bytes, stream);
    if (st != GSR_OK) return st;
    SortArgs sa;
    sa.num = 0;
    sa.d_num = curr_offset;
    sa.cap = key_capacity;
    sa.end_bit = 32 + bits_for((uint32_t)tiles);
    sa.compress_depth = true;
    sa.keys_in = keys_unsorted;
    sa.vals_in = values_unsorted;
    sa.keys_out = keys_sorted;
    sa.vals_out = values_sorted;
    sa.ws = workspace;
    sa.ws_bytes = workspace_bytes;
    if ((e = launch_sort(sa, s)) != cudaSuccess) return GSR_CUDA_ERROR;
    if ((e = launch_tile_ranges(0, curr_offset, key_capacity, tiles, keys_sorted, ranges, false, s)) != cudaSuccess)
        return GSR_CUDA_ERROR;
    TrainRenderArgs ra = {};
    ra.W = width;
    ra.H = height;
    ra.P = P;
    ra.d_num = curr_offset;
    ra.cap = key_capacity;
    ra.vals = values_sorted;
    ra.ranges = reinterpret_cast<const int2*>(ranges);
    ra.xy = reinterpret_cast<const float2*>(points_xy);
    ra.rgbd = reinterpret_cast<const float4*>(rgb_depth);
    ra.con = reinterpret_cast<const float4*>(conic_opacity);
    for (int k = 0; k < 3; k++) ra.bg[k] = bg_color[k];
    ra.image = image;
    ra.T_final = T_final;
    ra.n_tile = n_tile;
    e = launch_render_train(ra, false, s);
    return e == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
}

gsr_status gsr_train_backward(int P, const float* means, const float* log_scales, const float* quats,
                              const float* logits, const float* shs, int width, int height, const float* cam_pos,
                              const float* cam_rot, float focal_x, float focal_y, float z_far, float z_near,
                              const float* bg_color, const int32_t* curr_offset, int64_t key_capacity,
                              const uint32_t* values_sorted, const int32_t* ranges, const int32_t* n_tile,
                              const float* T_final, const float* points_xy, const float* rgb_depth,
                              const float* conic_opacity, const float* grad_image, float* grad_xy, float* grad_con,
                              float* grad_rgb, float* g_means, float* g_log_scales, float* g_quats, float* g_logits,
                              float* g_shs, int accumulate, gsr_stream_t stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (P < 0 || width <= 0 || height <= 0 || !cam_pos || !cam_rot || !bg_color || !curr_offset || !ranges ||
        !n_tile || !T_final || !grad_image || !grad_xy || !grad_con || !grad_rgb)
        return GSR_INVALID_ARG;
    if (P == 0) return GSR_OK;
    if (!means || !log_scales || !quats || !logits || !shs || !g_means || !g_log_scales || !g_quats || !g_logits ||
        !g_shs)
        return GSR_INVALID_ARG;
    cudaError_t e = cudaMemsetAsync(grad_xy, 0, sizeof(float) * 2 * (size_t)P, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(grad_con, 0, sizeof(float) * 4 * (size_t)P, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(grad_rgb, 0, sizeof(float) * 3 * (size_t)P, s);
    if (e != cudaSuccess) return GSR_CUDA_ERROR;
    TrainRenderArgs ra = {};
    ra.W = width;
    ra.H = height;
    ra.P = P;
    ra.d_num = curr_offset;
    ra.cap = key_capacity;
    ra.vals = values_sorted;
    ra.ranges = reinterpret_cast<const int2*>(ranges);
    ra.xy = reinterpret_cast<const float2*>(points_xy);
    ra.rgbd = reinterpret_cast<const float4*>(rgb_depth);
    ra.con = reinterpret_cast<const float4*>(conic_opacity);
    for (int k = 0; k < 3; k++) ra.bg[k] = bg_color[k];
    ra.T_final = const_cast<float*>(T_final);
    ra.n_tile = const_cast<int32_t*>(n_tile);
    ra.grad_image = grad_image;
    ra.grad_xy = grad_xy;
    ra.grad_con = grad_con;
    ra.grad_rgb = grad_rgb;
    if ((e = launch_render_train(ra, true, s)) != cudaSuccess) return GSR_CUDA_ERROR;
    PreBackArgs pa;
    pa.P = P;
    pa.means = means;
    pa.log_scales = log_scales;
    pa.quats = quats;
    pa.logits = logits;
    pa.shs = shs;
    pa.cam = adj_camera(width, height, cam_pos, cam_rot, focal_x, focal_y, z_far, z_near);
    pa.gxy = grad_xy;
    pa.gcon = grad_con;
    pa.grgb = grad_rgb;
    pa.g_means = g_means;
    pa.g_log_scales = g_log_scales;
    pa.g_quats = g_quats;
    pa.g_logits = g_logits;
    pa.g_shs = g_shs;
    pa.accumulate = accumulate;
    k_preprocess_backward<<<div_up(P, 128), 128, 0, s>>>(pa);
    return cudaGetLastError() == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
}

size_t gsr_train_views_scratch_bytes(int n_views)
{
    if (n_views <= 0 || n_views > 32767) return 0;
    return ((size_t)n_views * sizeof(PreprocessParams) + 255) & ~(size_t)255;
}

gsr_status gsr_train_forward_views(int P, const float* means, const float* log_scales, const float* quats,
                                   const float* logits, const float* shs, int n_views, int width, int height,
                                   const float* cam_pos, const float* cam_rot, const float* cam_intr,
                                   const float* bg_color, float* opacity, float* cov3d, void* view_scratch,
                                   size_t view_scratch_bytes, int32_t* curr_offset, void* workspace,
                                   size_t workspace_bytes, uint64_t* keys_unsorted, uint32_t* values_unsorted,
                                   uint64_t* keys_sorted, uint32_t* values_sorted, int64_t key_capacity,
                                   float* points_xy, float* rgb_depth, float* conic_opacity, int32_t* ranges,
                                   int32_t* n_tile, float* T_final, float* image, int flags, gsr_stream_t stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (P < 0 || n_views <= 0 || width <= 0 || height <= 0 || !cam_pos || !cam_rot || !cam_intr || !bg_color ||
        !curr_offset || !workspace || !ranges || !n_tile || !T_final || !image || !opacity || !cov3d ||
        !view_scratch || (flags & ~GSR_QUAD_KEYS) != 0)
        return GSR_INVALID_ARG;
    const bool quad = (flags & GSR_QUAD_KEYS) != 0;
    if (quad && (long long)P * n_views > (long long)kQuadGidMask + 1) return GSR_INVALID_ARG;
    if (P > 0 && (!means || !log_scales || !quats || !logits || !shs || !points_xy || !rgb_depth || !conic_opacity))
        return GSR_INVALID_ARG;
    if (view_scratch_bytes < gsr_train_views_scratch_bytes(n_views)) return GSR_INVALID_ARG;
    if (workspace_bytes < sort_workspace_bytes(key_capacity) || key_capacity >= (1LL << 30)) return GSR_INVALID_ARG;
    const int tiles = div_up(width, 16) * div_up(height, 16);
    // values carry view * P + Gaussian; key tile ids view * kt + tile (or quad)
    if ((long long)P * n_views >= (1LL << 31) || (long long)tiles * n_views >= (1LL << 30)) return GSR_INVALID_ARG;
    const int kt = quad ? quad_cols(div_up(width, 16)) * quad_cols(div_up(height, 16)) : tiles;
    cudaError_t e = launch_scene_prepare(P, log_scales, quats, logits, opacity, cov3d, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(workspace, 0, sizeof(uint32_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(curr_offset, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return GSR_CUDA_ERROR;
    // every view's parameter block, as the single-view preprocess fills it,
    // with its rows at view * P and its tiles at view * tiles
    PreprocessParams* d_params = reinterpret_cast<PreprocessParams*>(view_scratch);
    std::vector<PreprocessParams> hp((size_t)n_views);
    for (int v = 0; v < n_views; v++) {
        const float* in = cam_intr + 4 * (size_t)v;  // focal_x, focal_y, z_far, z_near
        const size_t r = (size_t)v * P;
        const gsr_status st = preprocess_params(hp[v], P, means, shs, opacity, cov3d, width, height, 16, 16,
                                                cam_pos + 3 * (size_t)v, cam_rot + 9 * (size_t)v, in[0], in[1], in[2],
                                                in[3], points_xy + 2 * r, rgb_depth + 4 * r, conic_opacity + 4 * r,
                                                keys_unsorted, values_unsorted, key_capacity, curr_offset, workspace,
                                                workspace_bytes);
        if (st != GSR_OK) return st;
        if (hp[v].mq.capacity <= 0) return GSR_INVALID_ARG;
        hp[v].gid_base = (int)r;
        hp[v].tile_base = v * kt;
        hp[v].views = d_params;
        hp[v].quad = quad ? 1 : 0;
    }
    if (P == 0) {
        // no Gaussian: no key, and every pixel is the background
        e = cudaMemsetAsync(ranges, 0, sizeof(int32_t) * 2 * (size_t)kt * n_views, s);
    } else {
        PreprocessParams base = hp[0];
        base.n_views = n_views;
        base.interleave = 1;  // every view has the scene's P
        // a pageable source is staged before the call returns
        e = cudaMemcpyAsync(d_params, hp.data(), sizeof(PreprocessParams) * (size_t)n_views, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = launch_preprocess_views(base, n_views, n_views * div_up(P, 256), false, s);
        if (e != cudaSuccess) return GSR_CUDA_ERROR;
        SortArgs sa;
        sa.num = 0;
        sa.d_num = curr_offset;
        sa.cap = key_capacity;
        sa.end_bit = 32 + bits_for((uint32_t)(kt * n_views));
        sa.compress_depth = true;
        sa.keys_in = keys_unsorted;
        sa.vals_in = values_unsorted;
        sa.keys_out = keys_sorted;
        sa.vals_out = values_sorted;
        sa.ws = workspace;
        sa.ws_bytes = workspace_bytes;
        if ((e = launch_sort(sa, s)) != cudaSuccess) return GSR_CUDA_ERROR;
        e = launch_tile_ranges(0, curr_offset, key_capacity, kt * n_views, keys_sorted, ranges, false, s);
    }
    if (e != cudaSuccess) return GSR_CUDA_ERROR;
    TrainRenderArgs ra = {};
    ra.W = width;
    ra.H = height;
    ra.P = P * n_views;
    ra.n_views = n_views;
    ra.quad = quad ? 1 : 0;
    ra.d_num = curr_offset;
    ra.cap = key_capacity;
    ra.vals = values_sorted;
    ra.ranges = reinterpret_cast<const int2*>(ranges);
    ra.xy = reinterpret_cast<const float2*>(points_xy);
    ra.rgbd = reinterpret_cast<const float4*>(rgb_depth);
    ra.con = reinterpret_cast<const float4*>(conic_opacity);
    for (int k = 0; k < 3; k++) ra.bg[k] = bg_color[k];
    ra.image = image;
    ra.T_final = T_final;
    ra.n_tile = n_tile;
    e = launch_render_train(ra, false, s);
    return e == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
}

gsr_status gsr_train_backward_views(int P, const float* means, const float* log_scales, const float* quats,
                                    const float* logits, const float* shs, int n_views, int width, int height,
                                    const float* cam_pos, const float* cam_rot, const float* cam_intr,
                                    const float* bg_color, const int32_t* curr_offset, int64_t key_capacity,
                                    const uint32_t* values_sorted, const int32_t* ranges, const int32_t* n_tile,
                                    const float* T_final, const float* points_xy, const float* rgb_depth,
                                    const float* conic_opacity, const float* grad_image, float* grad_feat,
                                    float* g_means, float* g_log_scales, float* g_quats, float* g_logits,
                                    float* g_shs, int accumulate, int flags, gsr_stream_t stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (P < 0 || n_views <= 0 || width <= 0 || height <= 0 || !cam_pos || !cam_rot || !cam_intr || !bg_color ||
        !curr_offset || !ranges || !n_tile || !T_final || !grad_image || !grad_feat || (flags & ~GSR_QUAD_KEYS) != 0)
        return GSR_INVALID_ARG;
    const bool quad = (flags & GSR_QUAD_KEYS) != 0;
    if (quad && (long long)P * n_views > (long long)kQuadGidMask + 1) return GSR_INVALID_ARG;
    if ((reinterpret_cast<uintptr_t>(grad_feat) & 15u) != 0) return GSR_INVALID_ARG;  // 16-byte atomics
    const int tiles = div_up(width, 16) * div_up(height, 16);
    if ((long long)P * n_views >= (1LL << 31) || (long long)tiles * n_views >= (1LL << 30)) return GSR_INVALID_ARG;
    if (P == 0) return GSR_OK;
    if (!means || !log_scales || !quats || !logits || !shs || !g_means || !g_log_scales || !g_quats || !g_logits ||
        !g_shs || !values_sorted || !points_xy || !rgb_depth || !conic_opacity)
        return GSR_INVALID_ARG;
    const size_t rows = (size_t)P * n_views;
    cudaError_t e = cudaMemsetAsync(grad_feat, 0, sizeof(float) * 12 * rows, s);
    if (e != cudaSuccess) return GSR_CUDA_ERROR;
    TrainRenderArgs ra = {};
    ra.W = width;
    ra.H = height;
    ra.P = (int)rows;
    ra.n_views = n_views;
    ra.quad = quad ? 1 : 0;
    ra.d_num = curr_offset;
    ra.cap = key_capacity;
    ra.vals = values_sorted;
    ra.ranges = reinterpret_cast<const int2*>(ranges);
    ra.xy = reinterpret_cast<const float2*>(points_xy);
    ra.rgbd = reinterpret_cast<const float4*>(rgb_depth);
    ra.con = reinterpret_cast<const float4*>(conic_opacity);
    for (int k = 0; k < 3; k++) ra.bg[k] = bg_color[k];
    ra.T_final = const_cast<float*>(T_final);
    ra.n_tile = const_cast<int32_t*>(n_tile);
    ra.grad_image = grad_image;
    ra.grad_rec = grad_feat;
    if ((e = launch_render_train(ra, true, s)) != cudaSuccess) return GSR_CUDA_ERROR;
    for (int v0 = 0; v0 < n_views; v0 += kAdjViews) {
        PreBackViewsArgs pa;
        pa.P = P;
        pa.n_views = std::min(kAdjViews, n_views - v0);
        pa.means = means;
        pa.log_scales = log_scales;
        pa.quats = quats;
        pa.logits = logits;
        pa.shs = shs;
        for (int k = 0; k < pa.n_views; k++) {
            const int v = v0 + k;
            const float* in = cam_intr + 4 * (size_t)v;
            pa.cam[k] = adj_camera(width, height, cam_pos + 3 * (size_t)v, cam_rot + 9 * (size_t)v, in[0], in[1],
                                   in[2], in[3]);
        }
        pa.grec = reinterpret_cast<const float4*>(grad_feat) + 3 * (size_t)v0 * P;
        pa.g_means = g_means;
        pa.g_log_scales = g_log_scales;
        pa.g_quats = g_quats;
        pa.g_logits = g_logits;
        pa.g_shs = g_shs;
        pa.accumulate = (accumulate || v0 > 0) ? 1 : 0;
        k_preprocess_backward_views<<<div_up(P, 128), 128, 0, s>>>(pa);
        if (cudaGetLastError() != cudaSuccess) return GSR_CUDA_ERROR;
    }
    return GSR_OK;
}

}  // extern "C"
