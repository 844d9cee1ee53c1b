// Scene preparation and preprocess (projection, EWA conic, SH colour, culling,
// tile-key emission) for sm_103a.
//
// The arithmetic of the geometry, the SH colour and the tile tests follows
// the reference's expressions operation for operation
// (csrc/cuda_rasterizer/preprocess.cu:78-311, 354-413) and is compiled with
// the same fast-math flags, so that the emitted (tile, depth) keys agree
// with the reference build bit for bit.  The kernel structure is this
// library's own: 8 warps per CTA, each warp owns 32 consecutive Gaussians,
// and keys are staged per warp in shared memory and flushed with one global
// atomic per flush instead of one per 32-wide emission step.
#include <algorithm>

#include "gsr_internal.h"

namespace gsr {
namespace {

// ---------------------------------------------------------------------------
// Tiny vector / matrix types with the component semantics of the GLM calls in
// the reference (column-major mat3, left-to-right sums of products).

struct V3 {
    float x, y, z;
    // member form so that it also applies to temporaries, as glm's does
    __device__ __forceinline__ V3& operator+=(float s)
    {
        x += s;
        y += s;
        z += s;
        return *this;
    }
};
__device__ __forceinline__ V3 operator*(float s, V3 v) { return {s * v.x, s * v.y, s * v.z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }

struct M3 {
    float m[3][3];  // m[column][row]
};

__device__ __forceinline__ M3 m3_mul(const M3& a, const M3& b)
{
    M3 r;
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int k = 0; k < 3; k++) r.m[c][k] = a.m[0][k] * b.m[c][0] + a.m[1][k] * b.m[c][1] + a.m[2][k] * b.m[c][2];
    return r;
}

__device__ __forceinline__ M3 m3_transpose(const M3& a)
{
    M3 r;
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int k = 0; k < 3; k++) r.m[c][k] = a.m[k][c];
    return r;
}

__device__ __forceinline__ M3 m3_cols(float a0, float a1, float a2, float b0, float b1, float b2, float c0, float c1,
                                      float c2)
{
    M3 r;
    r.m[0][0] = a0; r.m[0][1] = a1; r.m[0][2] = a2;
    r.m[1][0] = b0; r.m[1][1] = b1; r.m[1][2] = b2;
    r.m[2][0] = c0; r.m[2][1] = c1; r.m[2][2] = c2;
    return r;
}

// Constants of preprocess.cu:13-38.
constexpr float kLog2e = 1.4426950216293334961f;
constexpr float kLn2 = 0.69314718055f;
constexpr float kCutoff = 8.0f;
constexpr float kBMinSq = 0.09f;
constexpr float kOThin = 0.5f;
#define GSR_SH_C0 0.28209479177387814f
#define GSR_SH_C1 0.4886025119029199f
#define GSR_SH_C2_0 1.0925484305920792f
#define GSR_SH_C2_1 (-1.0925484305920792f)
#define GSR_SH_C2_2 0.31539156525252005f
#define GSR_SH_C2_3 (-1.0925484305920792f)
#define GSR_SH_C2_4 0.5462742152960396f
#define GSR_SH_C3_0 (-0.5900435899266435f)
#define GSR_SH_C3_1 2.890611442640554f
#define GSR_SH_C3_2 (-0.4570457994644658f)
#define GSR_SH_C3_3 0.3731763325901154f
#define GSR_SH_C3_4 (-0.4570457994644658f)
#define GSR_SH_C3_5 1.445305721320277f
#define GSR_SH_C3_6 (-0.5900435899266435f)

__device__ __forceinline__ float ndc_to_pix(float v, int S) { return ((v + 1.0) * S - 1.0) * 0.5; }

__device__ __forceinline__ float3 xform43(V3 p, const float* m)
{
    return {m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12], m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13],
            m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14]};
}

__device__ __forceinline__ float4 xform44(V3 p, const float* m)
{
    return {m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12], m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13],
            m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14], m[3] * p.x + m[7] * p.y + m[11] * p.z + m[15]};
}

// EWA projection of the 3D covariance (Zwicker et al. 2002, eqs. 29/31) with
// the 1.3*tan(fov) clamp and the +0.3 low-pass; same steps as
// preprocess.cu:117-157.
__device__ __forceinline__ float3 cov2d(V3 p, float fx, float fy, float tanx, float tany, const float* s,
                                        const float* vm)
{
    float3 t = xform43(p, vm);
    const float limx = 1.3f * tanx;
    const float limy = 1.3f * tany;
    const float txtz = t.x / t.z;
    const float tytz = t.y / t.z;
    t.x = fminf(limx, fmaxf(-limx, txtz)) * t.z;
    t.y = fminf(limy, fmaxf(-limy, tytz)) * t.z;
    M3 J = m3_cols(fx / t.z, 0.0f, -(fx * t.x) / (t.z * t.z), 0.0f, fy / t.z, -(fy * t.y) / (t.z * t.z), 0, 0, 0);
    M3 W = m3_cols(vm[0], vm[4], vm[8], vm[1], vm[5], vm[9], vm[2], vm[6], vm[10]);
    M3 T = m3_mul(W, J);
    M3 V = m3_cols(s[0], s[1], s[2], s[1], s[3], s[4], s[2], s[4], s[5]);
    M3 cov = m3_mul(m3_mul(m3_transpose(T), m3_transpose(V)), T);
    cov.m[0][0] += 0.3f;
    cov.m[1][1] += 0.3f;
    return {cov.m[0][0], cov.m[0][1], cov.m[1][1]};
}

// Degree-3 SH colour: +0.5 bias, clamp at 0 only (preprocess.cu:159-255).
template <bool HALF>
__device__ __forceinline__ V3 sh_color(int idx, V3 p, V3 cam, const void* shs)
{
    V3 dir = p - cam;
    float l2 = dir.x * dir.x + dir.y * dir.y + dir.z * dir.z;
    float r = rsqrt_approx(l2);
    dir.x *= r;
    dir.y *= r;
    dir.z *= r;
    V3 v[16];
    if (HALF) {
        const uint4* b4 = reinterpret_cast<const uint4*>(reinterpret_cast<const __half*>(shs) + (size_t)idx * 48);
        uint4 raw[6];
#pragma unroll
        for (int k = 0; k < 6; k++) raw[k] = __ldg(b4 + k);
        const __half* h = reinterpret_cast<const __half*>(raw);
#pragma unroll
        for (int k = 0; k < 16; k++) v[k] = {__half2float(h[3 * k]), __half2float(h[3 * k + 1]), __half2float(h[3 * k + 2])};
    } else {
        const float4* b4 = reinterpret_cast<const float4*>(reinterpret_cast<const float*>(shs) + (size_t)idx * 48);
        float4 raw[12];
#pragma unroll
        for (int k = 0; k < 12; k++) raw[k] = __ldg(b4 + k);
        const float* f = reinterpret_cast<const float*>(raw);
#pragma unroll
        for (int k = 0; k < 16; k++) v[k] = {f[3 * k], f[3 * k + 1], f[3 * k + 2]};
    }
    V3 result = GSR_SH_C0 * v[0] += 0.5f;
    float x = dir.x, y = dir.y, z = dir.z;
    result = result - GSR_SH_C1 * y * v[1] + GSR_SH_C1 * z * v[2] - GSR_SH_C1 * x * v[3];
    float xx = x * x, yy = y * y, zz = z * z;
    float xy = x * y, yz = y * z, xz = x * z;
    result = result + GSR_SH_C2_0 * xy * v[4] + GSR_SH_C2_1 * yz * v[5] +
             GSR_SH_C2_2 * (2.0f * zz - xx - yy) * v[6] + GSR_SH_C2_3 * xz * v[7] + GSR_SH_C2_4 * (xx - yy) * v[8];
    result = result + GSR_SH_C3_0 * y * (3.0f * xx - yy) * v[9] + GSR_SH_C3_1 * xy * z * v[10] +
             GSR_SH_C3_2 * y * (4.0f * zz - xx - yy) * v[11] +
             GSR_SH_C3_3 * z * (2.0f * zz - 3.0f * xx - 3.0f * yy) * v[12] +
             GSR_SH_C3_4 * x * (4.0f * zz - xx - yy) * v[13] + GSR_SH_C3_5 * z * (xx - yy) * v[14] +
             GSR_SH_C3_6 * x * (xx - 3.0f * yy) * v[15];
    result.x = fmaxf(result.x, 0.0f);
    result.y = fmaxf(result.y, 0.0f);
    result.z = fmaxf(result.z, 0.0f);
    return result;
}

// Ellipse / tile-box tests (preprocess.cu:257-311).
//
// The arithmetic is written with explicit rounding intrinsics, one per
// operation of the reference's expressions, fused where those expressions
// contract under fast math (x * y + z -> fma(x, y, z); x * x - y * z ->
// fma(x, x, -(y * z))).  Left to the compiler, the fusion of the same
// expression can differ between the kernels that inline it, and a tile on
// the ellipse's edge then passes in one kernel and fails in another: the
// depth-first pipeline counts a Gaussian's tiles in one kernel and emits
// them in another, so the two must agree bit for bit.
__device__ __forceinline__ bool seg_hits_ellipse(float a, float b, float c, float d, float l, float r)
{
    const float two_a = __fmul_rn(2.0f, a);
    const float delta = __fmaf_rn(b, b, -__fmul_rn(__fmul_rn(4.0f, a), c));
    const float t1 = __fmaf_rn(__fsub_rn(l, d), two_a, b);
    const float t2 = __fmaf_rn(__fsub_rn(r, d), two_a, b);
    return delta >= 0.0f && (t1 <= 0.0f || __fmul_rn(t1, t1) <= delta) &&
           (t2 >= 0.0f || __fmul_rn(t2, t2) <= delta);
}

__device__ __forceinline__ bool box_hits_ellipse(int2 pmin, int2 pmax, float2 ctr, float3 con, float power)
{
    float a, b, c, dx, dy;
    const float w = __fmul_rn(2.0f, power);
    if (ctr.x * 2.0f < (float)(pmin.x + pmax.x)) dx = __fsub_rn(ctr.x, (float)pmin.x);
    else dx = __fsub_rn(ctr.x, (float)pmax.x);
    a = con.z;
    b = __fmul_rn(__fmul_rn(-2.0f, con.y), dx);
    c = __fmaf_rn(__fmul_rn(con.x, dx), dx, -w);
    if (seg_hits_ellipse(a, b, c, ctr.y, (float)pmin.y, (float)pmax.y)) return true;
    if (ctr.y * 2.0f < (float)(pmin.y + pmax.y)) dy = __fsub_rn(ctr.y, (float)pmin.y);
    else dy = __fsub_rn(ctr.y, (float)pmax.y);
    a = con.x;
    b = __fmul_rn(__fmul_rn(-2.0f, con.y), dy);
    c = __fmaf_rn(__fmul_rn(con.z, dy), dy, -w);
    return seg_hits_ellipse(a, b, c, ctr.x, (float)pmin.x, (float)pmax.x);
}

__device__ __forceinline__ bool box_has_centre(int2 pmin, int2 pmax, float2 c)
{
    return c.x >= pmin.x && c.x <= pmax.x && c.y >= pmin.y && c.y <= pmax.y;
}

__device__ __forceinline__ bool tile_hit(int x, int y, int bx, int by, float2 ctr, float3 con, float power)
{
    int2 pmin = {x * bx, y * by};
    int2 pmax = {pmin.x + bx - 1, pmin.y + by - 1};
    return box_has_centre(pmin, pmax, ctr) || (power > 0.0f && box_hits_ellipse(pmin, pmax, ctr, con, power));
}

// Tiles of quad (qx, qy) that lie in the Gaussian's rectangle [rmin, rmax)
// and pass tile_hit: bit (x & 1) | (y & 1) << 1 per hit tile.  These are
// exactly the tiles the per-tile emission would give keys.
__device__ __forceinline__ uint32_t quad_mask(int qx, int qy, int2 rmin, int2 rmax, int bx, int by, float2 ctr,
                                              float3 con, float power)
{
    uint32_t m = 0u;
#pragma unroll
    for (int s = 0; s < 4; s++) {
        const int x = 2 * qx + (s & 1), y = 2 * qy + (s >> 1);
        if (x >= rmin.x && x < rmax.x && y >= rmin.y && y < rmax.y && tile_hit(x, y, bx, by, ctr, con, power))
            m |= 1u << s;
    }
    return m;
}

// Quad-rectangle [q0, q1) covering tile columns (or rows) [t0, t1), t1 > t0.
__device__ __forceinline__ int quad_lo(int t0) { return t0 >> 1; }
__device__ __forceinline__ int quad_hi(int t1) { return ((t1 - 1) >> 1) + 1; }

// ---------------------------------------------------------------------------
// Per-warp key staging.  A warp appends up to 32 keys per step into its own
// shared-memory ring; when the next step could overflow it, the warp
// reserves space in the global key buffer with one atomicAdd and copies the
// staged keys out with coalesced stores.
constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr int kStage = 256;

struct Stage {
    uint64_t* k;
    uint32_t* v;
    int fill;
};

struct EmitOut {
    uint64_t* keys;
    uint32_t* vals;
    long long cap;
    int* counter;
};

__device__ __forceinline__ void stage_flush(Stage& s, const EmitOut& o, unsigned lane)
{
    __syncwarp();
    int base = 0;
    if (lane == 0) base = atomicAdd(o.counter, s.fill);
    base = __shfl_sync(GSR_FULL_MASK, base, 0);
    for (int i = lane; i < s.fill; i += 32) {
        long long pos = (long long)base + i;
        if (pos >= 0 && pos < o.cap) {  // a counter past 2^31 wraps: never write below the buffer
            o.keys[pos] = s.k[i];
            o.vals[pos] = s.v[i];
        }
    }
    __syncwarp();
    s.fill = 0;
}

__device__ __forceinline__ void stage_emit(Stage& s, const EmitOut& o, bool valid, uint64_t key, uint32_t val,
                                           unsigned lane)
{
    unsigned mask = __ballot_sync(GSR_FULL_MASK, valid);
    if (mask == 0) return;
    int n = __popc(mask);
    if (s.fill + n > kStage) stage_flush(s, o, lane);
    if (valid) {
        int slot = s.fill + __popc(mask & lanemask_lt());
        s.k[slot] = key;
        s.v[slot] = val;
    }
    s.fill += n;
}

// Dispatch thresholds (PreprocessParams::massive_area / huge_area; the
// defaults are kDefaultMassiveArea / kDefaultHugeArea): tile rectangles at
// least massive_area tiles large are queued for k_emit_massive, and of those
// the ones of at least huge_area tiles are swept by a whole CTA.  They only
// decide which scheme tests a rectangle's tiles, never which keys come out.

// Block-wide final flush of every warp's staged keys with one atomic per CTA.
__device__ __forceinline__ void block_flush(Stage& st, const EmitOut& out, int* s_fill, long long* s_base,
                                            unsigned lane, int warp)
{
    if (lane == 0) s_fill[warp] = st.fill;
    __syncthreads();
    if (warp == 0) {
        int f = lane < kWarps ? s_fill[lane] : 0;
        int incl = f;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            int n = __shfl_up_sync(GSR_FULL_MASK, incl, d);
            if ((int)lane >= d) incl += n;
        }
        int total = __shfl_sync(GSR_FULL_MASK, incl, 31);
        long long base = 0;
        if (lane == 0 && total > 0) base = atomicAdd(out.counter, total);
        base = __shfl_sync(GSR_FULL_MASK, base, 0);
        if (lane < kWarps) s_base[lane] = base + incl - f;
    }
    __syncthreads();
    const long long wb = s_base[warp];
    for (int i = lane; i < st.fill; i += 32) {
        long long pos = wb + i;
        if (pos >= 0 && pos < out.cap) {
            out.keys[pos] = st.k[i];
            out.vals[pos] = st.v[i];
        }
    }
    st.fill = 0;
}

// COUNT = false: emit (tile | depth, index) keys (the reference's single-pass
// pipeline).  COUNT = true: the depth-first pipeline's counting pass -- the
// same tests, but each Gaussian's number of hit tiles is counted and written
// with its depth and test geometry instead of keys.
//
// QUAD: keys name 2x2 groups of tiles, with the hit tiles as a mask in the
// value (PreprocessParams::quad), and the counting pass counts those quads;
// the tile rectangle, the dispatch and every tile test are the per-tile
// emission's.
template <bool HALF, bool COUNT, bool VIEWS, bool QUAD = false>
__global__ __launch_bounds__(kThreads, VIEWS ? 6 : 5) void k_preprocess(const __grid_constant__ PreprocessParams a0)
{
    // VIEWS: the views' blocks follow one another along the grid (parameter
    // blocks in device memory); a block past the last view has no work
    int vi = 0, lblock = (int)blockIdx.x;
    if (VIEWS && a0.interleave) {
        vi = (int)(blockIdx.x % (unsigned)a0.n_views);
        lblock = (int)(blockIdx.x / (unsigned)a0.n_views);
        if (lblock >= (a0.views[vi].P + kThreads - 1) / kThreads) return;
    } else if (VIEWS) {
        vi = -1;
        for (int u = 0, start = 0; u < a0.n_views; u++) {
            const int nb = (a0.views[u].P + kThreads - 1) / kThreads;
            if (lblock < start + nb) {
                vi = u;
                lblock -= start;
                break;
            }
            start += nb;
        }
        if (vi < 0) return;
    }
    const PreprocessParams& a = VIEWS ? a0.views[vi] : a0;
    const uint32_t view_tag = VIEWS ? ((uint32_t)vi << 16) : 0u;
    __shared__ uint64_t s_keys[COUNT ? 1 : kWarps][kStage];
    __shared__ uint32_t s_vals[COUNT ? 1 : kWarps][kStage];
    __shared__ int s_fill[kWarps];
    __shared__ long long s_base[kWarps];
    __shared__ uint32_t s_hit[kWarps];
    __shared__ int s_pref[kWarps][32];
    __shared__ uint32_t s_cnt[kWarps][32];

    const unsigned lane = threadIdx.x & 31u;
    const int warp = threadIdx.x >> 5;
    const int idx = lblock * kThreads + threadIdx.x;
    const int warp_first = idx - (int)lane;
    const int tx = lane & 7, ty = lane >> 3;  // 8x4 tile window of the massive path
    const int gridx = a.gx, gridy = a.gy;
    const int qgx = quad_cols(gridx);  // quads per row (QUAD)

    bool point_valid = false;
    V3 p_orig = {0.f, 0.f, 0.f};
    float3 p_view = {0.f, 0.f, 0.f};
    float2 point_xy = {0.f, 0.f};
    float3 conic = {0.f, 0.f, 0.f};
    float opacity = 0.f, power = 0.f, log2_opacity = 0.f;
    int width = 0, height = 0;
    int2 rect_min = {0, 0}, rect_max = {0, 0};

    if (idx < a.P) {
        do {
            p_orig = {__ldg(a.pos + 3 * (size_t)idx), __ldg(a.pos + 3 * (size_t)idx + 1),
                      __ldg(a.pos + 3 * (size_t)idx + 2)};
            p_view = xform43(p_orig, a.view);
            if (p_view.z <= 0.2f) break;
            opacity = __ldg(a.opacity + idx);
            float4 p_hom = xform44(p_orig, a.proj);
            float p_w = 1.0f / (p_hom.w + 0.0000001f);
            float3 p_proj = {p_hom.x * p_w, p_hom.y * p_w, p_hom.z * p_w};
            float s6[6];
            const float2* c2 = reinterpret_cast<const float2*>(a.cov3d + 6 * (size_t)idx);
            float2 c01 = __ldg(c2), c23 = __ldg(c2 + 1), c45 = __ldg(c2 + 2);
            s6[0] = c01.x; s6[1] = c01.y; s6[2] = c23.x; s6[3] = c23.y; s6[4] = c45.x; s6[5] = c45.y;
            float3 cov = cov2d(p_orig, a.fx, a.fy, a.tanx, a.tany, s6, a.view);
            float det = (cov.x * cov.z - cov.y * cov.y);
            float det_inv = 1.f / det;
            conic = {cov.z * det_inv, -cov.y * det_inv, cov.x * det_inv};
            log2_opacity = lg2_approx(opacity);
            power = kLn2 * kCutoff + kLn2 * log2_opacity;
            float trace = cov.x + cov.z;
            if (2.0f * det * power < kBMinSq * trace && opacity < kOThin) break;
            width = (int)(1.414214f * sqrt_approx(cov.x * power) + 1.0f);
            height = (int)(1.414214f * sqrt_approx(cov.z * power) + 1.0f);
            point_xy = {ndc_to_pix(p_proj.x, a.W), ndc_to_pix(p_proj.y, a.H)};
            rect_min = {min(gridx, max(0, (int)((point_xy.x - width) / (float)a.bx))),
                        min(gridy, max(0, (int)((point_xy.y - height) / (float)a.by)))};
            rect_max = {min(gridx, max(0, (int)((point_xy.x + width) / (float)a.bx) + 1)),
                        min(gridy, max(0, (int)((point_xy.y + height) / (float)a.by) + 1))};
            point_valid = (rect_max.x - rect_min.x) * (rect_max.y - rect_min.y) > 0;
        } while (false);
    }
    Stage st{s_keys[COUNT ? 0 : warp], s_vals[COUNT ? 0 : warp], 0};
    const EmitOut out{a.keys, a.vals, a.cap, a.counter};
    if (lane == 0) s_hit[warp] = 0u;
    s_cnt[warp][lane] = 0u;
    __syncwarp();
    const uint32_t depth_bits = __float_as_uint(p_view.z);
    const bool was_valid = point_valid;
    bool queued = false;

    // (1) single-tile Gaussians: one test per thread.
    const int area = (rect_max.x - rect_min.x) * (rect_max.y - rect_min.y);
    const bool single = point_valid && area == 1;
    {
        bool v = single && tile_hit(rect_min.x, rect_min.y, a.bx, a.by, point_xy, conic, power);
        if (COUNT) {
            if (v) s_cnt[warp][lane] = 1u;
        } else if (QUAD) {
            const uint32_t qt = (uint32_t)(a.tile_base + (rect_min.y >> 1) * qgx + (rect_min.x >> 1));
            const uint32_t bit = 1u << ((rect_min.x & 1) | ((rect_min.y & 1) << 1));
            stage_emit(st, out, v, ((uint64_t)qt << 32) | depth_bits, (uint32_t)(a.gid_base + idx) | (bit << kQuadShift),
                       lane);
        } else {
            uint64_t key = ((uint64_t)(uint32_t)(a.tile_base + rect_min.y * gridx + rect_min.x) << 32) | depth_bits;
            stage_emit(st, out, v, key, (uint32_t)(a.gid_base + idx), lane);
        }
        unsigned m = __ballot_sync(GSR_FULL_MASK, v);
        if (lane == 0 && m) atomicOr(&s_hit[warp], m);
    }
    point_valid = point_valid && !single;

    // (2) multi-tile Gaussians.  Rectangles of at least massive_area tiles go
    // to the massive queue, where a whole CTA tests them (k_emit_massive);
    // the rest form one flattened task pool per warp (the reference's
    // "fragmented" scheme, preprocess.cu:521-623).  If the queue is full, the
    // warp tests the Gaussian itself over an 8x4 tile window (the reference's
    // "massive" scheme, preprocess.cu:444-519).  Every scheme tests every
    // tile of the rectangle with the same test, so the key set is the same.
    bool massive = point_valid && area >= a.massive_area;
    {
        // huge rectangles first try the CTA-swept region, then the warp one
        int slot = -1;
        const bool want_huge = massive && area >= a.huge_area;
        const unsigned mh = __ballot_sync(GSR_FULL_MASK, want_huge);
        if (mh) {
            int base = 0;
            if (lane == 0) base = (int)atomicAdd(&a.mq.count[0], (uint32_t)__popc(mh));
            base = __shfl_sync(GSR_FULL_MASK, base, 0);
            const int s0 = base + __popc(mh & lanemask_lt());
            if (want_huge && s0 < a.mq.huge_capacity) slot = s0;
        }
        const bool want_large = massive && slot < 0;
        const unsigned ml = __ballot_sync(GSR_FULL_MASK, want_large);
        if (ml) {
            int base = 0;
            if (lane == 0) base = (int)atomicAdd(&a.mq.count[1], (uint32_t)__popc(ml));
            base = __shfl_sync(GSR_FULL_MASK, base, 0);
            const int s1 = base + __popc(ml & lanemask_lt());
            if (want_large && s1 < a.mq.capacity - a.mq.huge_capacity) slot = a.mq.huge_capacity + s1;
        }
        if (slot >= 0) {
            MassiveEntry e;
            e.ctr_power_depth = make_float4(point_xy.x, point_xy.y, power, p_view.z);
            e.conic_gid = make_float4(conic.x, conic.y, conic.z, __uint_as_float((uint32_t)(a.gid_base + idx)));
            // x0 < 2^16; the view index rides in the high half
            e.rect = make_int4((int)((uint32_t)rect_min.x | view_tag), rect_max.x, rect_min.y, rect_max.y);
            a.mq.entries[slot] = e;
            atomicOr(&s_hit[warp], 1u << lane);  // features are written for queued Gaussians
            point_valid = false;
            massive = false;
            queued = true;
        }
    }
    // queue overflow: the warp runs the Gaussian's whole rectangle itself
    unsigned todo = __ballot_sync(GSR_FULL_MASK, massive);
    while (todo) {
        const int i = __ffs(todo) - 1;
        todo &= todo - 1;
        const float2 c = {__shfl_sync(GSR_FULL_MASK, point_xy.x, i), __shfl_sync(GSR_FULL_MASK, point_xy.y, i)};
        const float3 q = {__shfl_sync(GSR_FULL_MASK, conic.x, i), __shfl_sync(GSR_FULL_MASK, conic.y, i),
                          __shfl_sync(GSR_FULL_MASK, conic.z, i)};
        const int x_lo = __shfl_sync(GSR_FULL_MASK, rect_min.x, i), y_lo = __shfl_sync(GSR_FULL_MASK, rect_min.y, i);
        const int x_hi = __shfl_sync(GSR_FULL_MASK, rect_max.x, i), y_hi = __shfl_sync(GSR_FULL_MASK, rect_max.y, i);
        const uint32_t db = __shfl_sync(GSR_FULL_MASK, depth_bits, i);
        const float pw = __shfl_sync(GSR_FULL_MASK, power, i);
        const uint32_t gid = (uint32_t)(a.gid_base + warp_first + i);
        if (QUAD) {
            const int qx_lo = quad_lo(x_lo), qx_hi = quad_hi(x_hi), qy_lo = quad_lo(y_lo), qy_hi = quad_hi(y_hi);
            for (int y0 = qy_lo; y0 < qy_hi; y0 += 4) {
                const int qy = y0 + ty;
                for (int x0 = qx_lo; x0 < qx_hi; x0 += 8) {
                    const int qx = x0 + tx;
                    const uint32_t m = (qy < qy_hi && qx < qx_hi)
                                           ? quad_mask(qx, qy, make_int2(x_lo, y_lo), make_int2(x_hi, y_hi), a.bx,
                                                       a.by, c, q, pw)
                                           : 0u;
                    if (COUNT) {
                        const unsigned mm = __ballot_sync(GSR_FULL_MASK, m != 0u);
                        if (lane == 0) s_cnt[warp][i] += __popc(mm);
                    } else {
                        const uint64_t key = ((uint64_t)(uint32_t)(a.tile_base + qy * qgx + qx) << 32) | db;
                        stage_emit(st, out, m != 0u, key, gid | (m << kQuadShift), lane);
                    }
                }
            }
        } else {
            for (int y0 = y_lo; y0 < y_hi; y0 += 4) {
                const int y = y0 + ty;
                for (int x0 = x_lo; x0 < x_hi; x0 += 8) {
                    const int x = x0 + tx;
                    bool v = y < y_hi && x < x_hi && tile_hit(x, y, a.bx, a.by, c, q, pw);
                    if (COUNT) {
                        const unsigned m = __ballot_sync(GSR_FULL_MASK, v);
                        if (lane == 0) s_cnt[warp][i] += __popc(m);
                    } else {
                        uint64_t key = ((uint64_t)(uint32_t)(a.tile_base + y * gridx + x) << 32) | db;
                        stage_emit(st, out, v, key, gid, lane);
                    }
                }
            }
        }
        if (lane == 0) atomicOr(&s_hit[warp], 1u << i);
    }
    point_valid = point_valid && !massive;

    // tasks of the pool: the rectangle's tiles, or (QUAD) the quads covering it
    const int my_tiles = !point_valid ? 0
                         : QUAD      ? (quad_hi(rect_max.x) - quad_lo(rect_min.x)) *
                                      (quad_hi(rect_max.y) - quad_lo(rect_min.y))
                                     : area;
    const unsigned multi = __ballot_sync(GSR_FULL_MASK, point_valid);
    if (multi) {
        int prefix = my_tiles;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            int n = __shfl_up_sync(GSR_FULL_MASK, prefix, d);
            if ((int)lane >= d) prefix += n;
        }
        const int total = __shfl_sync(GSR_FULL_MASK, prefix, 31);
        s_pref[warp][lane] = prefix;  // inclusive prefix of the tile counts
        __syncwarp();
        prefix -= my_tiles;
        for (int base = 0; base < total; base += 32) {
            const int task = base + (int)lane;
            const bool task_ok = task < total;
            // owner = first lane whose inclusive prefix exceeds the task index
            int lo = 0, hi = 31;
#pragma unroll
            for (int step = 0; step < 5; step++) {
                const int mid = (lo + hi) >> 1;
                if (s_pref[warp][mid] > task) hi = mid;
                else lo = mid + 1;
            }
            const int owner = task_ok ? lo : __ffs(multi) - 1;
            const int ox = __shfl_sync(GSR_FULL_MASK, rect_min.x, owner);
            const int oy = __shfl_sync(GSR_FULL_MASK, rect_min.y, owner);
            const int ow = __shfl_sync(GSR_FULL_MASK, rect_max.x, owner) - ox;
            const int op = __shfl_sync(GSR_FULL_MASK, prefix, owner);
            const float2 c = {__shfl_sync(GSR_FULL_MASK, point_xy.x, owner),
                              __shfl_sync(GSR_FULL_MASK, point_xy.y, owner)};
            const float3 q = {__shfl_sync(GSR_FULL_MASK, conic.x, owner), __shfl_sync(GSR_FULL_MASK, conic.y, owner),
                              __shfl_sync(GSR_FULL_MASK, conic.z, owner)};
            const float pw = __shfl_sync(GSR_FULL_MASK, power, owner);
            const uint32_t db = __shfl_sync(GSR_FULL_MASK, depth_bits, owner);
            int x = 0, y = 0;
            bool v = false;
            uint32_t qm = 0u;
            if (QUAD) {
                const int oy1 = __shfl_sync(GSR_FULL_MASK, rect_max.y, owner);
                const int oqx = quad_lo(ox), oqw = quad_hi(ox + ow) - oqx;
                if (task_ok) {
                    const int local = task - op;
                    const int row = oqw > 0 ? local / oqw : 0;
                    x = oqx + (local - row * oqw);
                    y = quad_lo(oy) + row;
                    qm = quad_mask(x, y, make_int2(ox, oy), make_int2(ox + ow, oy1), a.bx, a.by, c, q, pw);
                    v = qm != 0u;
                }
            } else if (task_ok) {
                const int local = task - op;
                const int row = ow > 0 ? local / ow : 0;
                x = ox + (local - row * ow);
                y = oy + row;
                v = tile_hit(x, y, a.bx, a.by, c, q, pw);
            }
            if (COUNT) {
                if (v) atomicAdd(&s_cnt[warp][owner], 1u);
            } else if (QUAD) {
                const uint64_t key = ((uint64_t)(uint32_t)(a.tile_base + y * qgx + x) << 32) | db;
                stage_emit(st, out, v, key, (uint32_t)(a.gid_base + warp_first + owner) | (qm << kQuadShift), lane);
            } else {
                uint64_t key = ((uint64_t)(uint32_t)(a.tile_base + y * gridx + x) << 32) | db;
                stage_emit(st, out, v, key, (uint32_t)(a.gid_base + warp_first + owner), lane);
            }
            if (v) atomicOr(&s_hit[warp], 1u << owner);
        }
    }
    __syncwarp();

    // (3) render features for every Gaussian that emitted at least one key.
    const bool emitted = (s_hit[warp] >> lane) & 1u;
    if (a.mq.depth_hi) {
        const uint32_t m = __reduce_max_sync(GSR_FULL_MASK, emitted ? depth_bits : 0u);
        if (lane == 0 && m) atomicMax(a.mq.depth_hi, m);
    }
    if (emitted) {
        a.points_xy[idx] = point_xy;
        a.conic_opacity[idx] = make_float4((-0.5f * kLog2e) * conic.x, -kLog2e * conic.y, (-0.5f * kLog2e) * conic.z,
                                           log2_opacity);
        V3 cam = {a.campos[0], a.campos[1], a.campos[2]};
        V3 col = sh_color<HALF>(idx, p_orig, cam, a.shs);
        a.rgb_depth[idx] = make_float4(col.x, col.y, col.z, p_view.z);
    }

    if (COUNT) {
        // The reference's ES layout writes a Gaussian's depth (and records)
        // only where its pass A marks the Gaussian valid, which depends on
        // that pass's warp-level dispatch (preprocess.cu:800-874, 957-985):
        // always for a one-tile rectangle; for larger ones always on its
        // pooled path, but on its per-Gaussian path (taken when the warp
        // holds at most two multi-tile Gaussians or one of at least 32
        // tiles) only when a tile was hit.  The others get depth FLT_MAX.
        // Both passes give a warp the same 32 consecutive Gaussians, and the
        // ES layout runs without the large-Gaussian queue, so s_cnt holds the
        // final counts here.
        bool ref_valid = false;
        if (a.df.ref_layout) {  // uniform over the warp
            const bool multi_g = was_valid && area > 1;
            const unsigned mg = __ballot_sync(GSR_FULL_MASK, multi_g);
            const int max_area = __reduce_max_sync(GSR_FULL_MASK, multi_g ? area : 0);
            const bool per_gaussian_path = __popc(mg) <= 2 || max_area >= 32;
            ref_valid = (was_valid && area == 1) || (multi_g && (!per_gaussian_path || s_cnt[warp][lane] > 0u));
        }
        // (4') records of the counting pass (queued Gaussians get their count
        // from the massive kernel, which runs next)
        if (idx < a.P) {
            a.df.count[idx] = was_valid ? s_cnt[warp][lane] : 0u;
            if (a.df.ref_layout && !ref_valid) a.df.dkey[idx] = 0x7F7FFFFFu;  // FLT_MAX (preprocess.cu:983)
            if (was_valid && (!a.df.ref_layout || ref_valid)) a.df.dkey[idx] = depth_bits;
            if (was_valid) {
                a.df.geo[idx] = make_float4(conic.x, conic.y, conic.z, power);
                if (a.df.ref_layout)  // (rect_min, rect_max) packed as (x | y << 16), preprocess.cu:975-977
                    a.df.rect[idx] = make_int2((int)((uint32_t)rect_min.x | ((uint32_t)rect_min.y << 16)),
                                               (int)((uint32_t)rect_max.x | ((uint32_t)rect_max.y << 16)));
                else
                    a.df.rect[idx] = make_int2((int)((uint32_t)rect_min.x | ((uint32_t)rect_max.x << 16)),
                                               (int)((uint32_t)rect_min.y | ((uint32_t)rect_max.y << 16) |
                                                     (queued ? 0x80000000u : 0u)));
            }
        }
    } else {
        // (4) block-wide final flush: one atomic per CTA.
        block_flush(st, out, s_fill, s_base, lane, warp);
    }
}

// ---------------------------------------------------------------------------
// Queued Gaussians with large tile rectangles (k_emit_massive).  For a
// well-conditioned ellipse only the tiles of each tile row that lie within a
// margin of the ellipse's x-extent over that row get the exact test; tiles
// farther out cannot pass it.
constexpr int kMaxBandRows = 1024;  // tile rows of a CTA-swept rectangle that get candidate bands

// Ellipse A dx^2 + 2B dx dy + C dy^2 <= w (w = 2 power) in float.
//
// Which tiles can pass the exact test.  In exact arithmetic the test
// (box_has_centre / box_hits_ellipse) only accepts tiles whose box meets the
// ellipse.  In float it can also accept a tile just outside.  On a box edge
// at offset dx from the centre, the test accepts a point of the edge where
// the computed quadratic is <= 0; the computed discriminant errs by a few
// 2^-24 of its terms' size, (B^2 + AC) dx^2 + C w, so every accepted point
// satisfies Q <= w (1 + k u (1 + kappa)), with u = 2^-24, kappa = 2AC / det
// >= (B^2 + AC) / det and k about 10 (the same holds for the horizontal
// edge).  The candidate bands are therefore the exact row extents of the
// ellipse inflated to w (1 + tau), tau = 64 u (1 + kappa), plus half a pixel
// and a relative 1e-5 for the rounding of the band arithmetic itself and of
// pixel coordinates.
//
// det = AC - B^2 is formed with a single rounding (Kahan's fused difference
// of products), and the half-width at height dy as sqrt(det (dymax - dy)
// (dymax + dy)) / A, which does not cancel near the top and bottom, so every
// extent carries a few ulp of relative error.  Ill-conditioned ellipses
// (det <= 1e-6 AC) and non-finite values get every tile of the rectangle
// tested.
struct Band {
    float B, inv_a, det, dymax, dxmax, dyr, cx, cy, m;
    bool ok;
};

__device__ __forceinline__ Band make_band(float3 q, float power, float2 c)
{
    Band b;
    const float A = q.x, B = q.y, C = q.z, w = 2.0f * power;
    const float bb = B * B;
    const float det = fmaf(A, C, -bb) + fmaf(-B, B, bb);
    const float kappa = 2.0f * (A * C) / det;
    const float wb = w * (1.0f + 64.0f * 5.9604645e-8f * (1.0f + kappa));  // inflated for the test's rounding
    b.B = B;
    b.inv_a = 1.0f / A;
    b.det = det;
    b.dymax = sqrtf(wb * A / det);
    b.dxmax = sqrtf(wb * C / det);
    b.dyr = -B * sqrtf(wb / (C * det));  // dy where the ellipse reaches its largest x
    b.cx = c.x;
    b.cy = c.y;
    b.m = 0.5f + 1e-5f * fmaxf(b.dxmax, b.dymax);
    b.ok = A > 0.0f && C > 0.0f && w > 0.0f && det > 1e-6f * (A * C) && b.dymax < 1e6f && b.dxmax < 1e6f &&
           fabsf(b.dyr) < 1e6f && fabsf(c.x) < 1e7f && fabsf(c.y) < 1e7f;
    return b;
}

// Candidate tile columns [c_lo, c_hi] of tile row `ty`: the ellipse's x-extent
// over the row's pixel band, widened by m pixels on every side.  False when
// the widened band misses the ellipse.
__device__ __forceinline__ bool band_columns(const Band& e, int ty, int by, int bx, int x_lo, int x_hi, int& c_lo,
                                             int& c_hi)
{
    const float p = fmaxf((float)(ty * by) - e.m - e.cy, -e.dymax);
    const float q = fminf((float)(ty * by + by - 1) + e.m - e.cy, e.dymax);
    if (!(p <= q)) return false;
    auto half = [&](float dy) {
        return sqrtf(e.det * fmaxf(0.0f, e.dymax - dy) * fmaxf(0.0f, e.dymax + dy)) * e.inv_a;
    };
    const float hp = half(p), hq = half(q);
    const float mp = -e.B * p * e.inv_a, mq = -e.B * q * e.inv_a;  // centre line of the ellipse at p, q
    const float xr = (e.dyr >= p && e.dyr <= q) ? e.dxmax : fmaxf(mp + hp, mq + hq);
    const float xl = (-e.dyr >= p && -e.dyr <= q) ? -e.dxmax : fminf(mp - hp, mq - hq);
    const float lo = floorf((e.cx + xl - e.m) / (float)bx), hi = floorf((e.cx + xr + e.m) / (float)bx);
    c_lo = (int)fmaxf((float)x_lo, lo);
    c_hi = (int)fminf((float)(x_hi - 1), hi);
    return c_lo <= c_hi;
}

// The CTA's flattened sweep of `rows` rows of candidate columns (s_band[r] =
// [lo, hi], empty when hi < lo): a block-wide prefix of the rows' counts
// into s_pref, then each warp takes 32 consecutive candidates at a time, so
// a narrow row shares a step with its neighbours instead of taking a step of
// its own.  step(valid, x, r) is called by all lanes of a warp together.
template <typename F>
__device__ __forceinline__ void sweep_flat_cta(int rows, const short2* s_band, int* s_pref, int* s_wsum,
                                               unsigned lane, int warp, F&& step)
{
    constexpr int kPer = kMaxBandRows / kThreads;  // rows per thread in the scan
    const int r0 = (int)threadIdx.x * kPer;
    int cnt[kPer];
    int local = 0;
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        const int r = r0 + k;
        cnt[k] = r < rows ? max(0, (int)s_band[r].y - (int)s_band[r].x + 1) : 0;
        local += cnt[k];
    }
    int incl = local;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(GSR_FULL_MASK, incl, d);
        if ((int)lane >= d) incl += t;
    }
    if (lane == 31) s_wsum[warp] = incl;
    __syncthreads();
    int run = incl - local, total = 0;
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
        if (w < warp) run += s_wsum[w];
        total += s_wsum[w];
    }
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        run += cnt[k];
        if (r0 + k < rows) s_pref[r0 + k] = run;  // inclusive prefix of the rows' counts
    }
    __syncthreads();
    for (int base = warp * 32; base < total; base += kWarps * 32) {
        const int task = base + (int)lane;
        // owner row: the first row whose inclusive prefix exceeds the task
        int lo = 0, hi = rows - 1;
#pragma unroll
        for (int it = 0; it < 10; it++) {  // 2^10 = kMaxBandRows
            if (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (s_pref[mid] > task) hi = mid;
                else lo = mid + 1;
            }
        }
        const short2 b = s_band[lo];
        const int x = (int)b.x + task - (s_pref[lo] - ((int)b.y - (int)b.x + 1));
        step(task < total, x, lo);
    }
}

// Sweep the tiles of one huge queued Gaussian with the whole CTA; on_step(v,
// x, y) is called by every lane of a warp together, v = the tile's exact test.
template <typename F>
__device__ __forceinline__ void sweep_cta(const MassiveEntry& me, const PreprocessParams& a, short2* s_band,
                                          int* s_pref, int* s_wsum, unsigned lane, int warp, F&& on_step)
{
    const float2 c = {me.ctr_power_depth.x, me.ctr_power_depth.y};
    const float pw = me.ctr_power_depth.z;
    const float3 q = {me.conic_gid.x, me.conic_gid.y, me.conic_gid.z};
    const int x_lo = me.rect.x & 0xFFFF, x_hi = me.rect.y, y_lo = me.rect.z, y_hi = me.rect.w;
    const int w = x_hi - x_lo;
    // every thread forms the same band from the same inputs: a uniform branch
    const Band eb = make_band(q, pw, c);
    if (eb.ok && (y_hi - y_lo) <= kMaxBandRows) {
        for (int r = threadIdx.x; r < y_hi - y_lo; r += kThreads) {
            int clo = 0, chi = -1;
            if (!band_columns(eb, y_lo + r, a.by, a.bx, x_lo, x_hi, clo, chi)) {
                clo = 0;
                chi = -1;
            }
            s_band[r] = make_short2((short)clo, (short)chi);
        }
        __syncthreads();
        sweep_flat_cta(y_hi - y_lo, s_band, s_pref, s_wsum, lane, warp, [&](bool valid, int x, int r) {
            on_step(valid && tile_hit(x, y_lo + r, a.bx, a.by, c, q, pw), x, y_lo + r);
        });
        __syncthreads();  // s_band, s_pref and on_step's shared counters are reused by the next entry
        return;
    }
    // Otherwise the CTA sweeps the rectangle in windows of (cols x rows)
    // tiles, cols a power of two fitted to the rectangle's width, so narrow
    // rectangles still fill the lanes and no per-tile integer division is
    // needed.
    int lg = 5;
    while (lg > 0 && (1 << (lg - 1)) >= w) lg--;
    const int cols = 1 << lg;              // columns per warp row
    const int rows_w = 32 >> lg;           // rows per warp
    const int rows_cta = rows_w * kWarps;  // rows per CTA step
    const int lx = (int)lane & (cols - 1);
    const int ly = warp * rows_w + ((int)lane >> lg);
    for (int wy = y_lo; wy < y_hi; wy += rows_cta) {
        const int y = wy + ly;
        for (int wx = x_lo; wx < x_hi; wx += cols) {
            const int x = wx + lx;
            const bool v = y < y_hi && x < x_hi && tile_hit(x, y, a.bx, a.by, c, q, pw);
            on_step(v, x, y);
        }
    }
    __syncthreads();  // on_step's shared counters are reused by the next entry
}

// Sweep the tiles of one large queued Gaussian with one warp: the candidate
// tiles of 32 rows at a time form one flattened task list, 32 tests per step.
template <typename F>
__device__ __forceinline__ void sweep_warp(const MassiveEntry& me, const PreprocessParams& a, unsigned lane,
                                           F&& on_step)
{
    const float2 c = {me.ctr_power_depth.x, me.ctr_power_depth.y};
    const float pw = me.ctr_power_depth.z;
    const float3 q = {me.conic_gid.x, me.conic_gid.y, me.conic_gid.z};
    const int x_lo = me.rect.x & 0xFFFF, x_hi = me.rect.y, y_lo = me.rect.z, y_hi = me.rect.w;
    const Band eb = make_band(q, pw, c);
    if (eb.ok) {
        for (int r0 = y_lo; r0 < y_hi; r0 += 32) {
            const int y = r0 + (int)lane;
            int clo = 0, n = 0;
            if (y < y_hi) {
                int chi = -1;
                if (band_columns(eb, y, a.by, a.bx, x_lo, x_hi, clo, chi)) n = chi - clo + 1;
            }
            int pref = n;  // inclusive prefix of the candidate counts
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int t = __shfl_up_sync(GSR_FULL_MASK, pref, d);
                if ((int)lane >= d) pref += t;
            }
            const int total = __shfl_sync(GSR_FULL_MASK, pref, 31);
            for (int base = 0; base < total; base += 32) {
                const int task = base + (int)lane;
                // owner row = first lane whose inclusive prefix exceeds the task
                int lo = 0, hi = 31;
#pragma unroll
                for (int step = 0; step < 5; step++) {
                    const int mid = (lo + hi) >> 1;
                    if (__shfl_sync(GSR_FULL_MASK, pref, mid) > task) hi = mid;
                    else lo = mid + 1;
                }
                const int o_pref = __shfl_sync(GSR_FULL_MASK, pref, lo);
                const int o_n = __shfl_sync(GSR_FULL_MASK, n, lo);
                const int o_clo = __shfl_sync(GSR_FULL_MASK, clo, lo);
                const int x = o_clo + task - (o_pref - o_n);
                const int yy = r0 + lo;
                const bool v = task < total && tile_hit(x, yy, a.bx, a.by, c, q, pw);
                on_step(v, x, yy);
            }
        }
        return;
    }
    const int w = x_hi - x_lo;
    const long long total = (long long)w * (long long)(y_hi - y_lo);
    for (long long base = 0; base < total; base += 32) {
        const long long t = base + lane;
        int x = 0, y = 0;
        bool v = false;
        if (t < total) {
            const int r = (int)(t / w);
            y = y_lo + r;
            x = x_lo + (int)(t - (long long)r * w);
            v = tile_hit(x, y, a.bx, a.by, c, q, pw);
        }
        on_step(v, x, y);
    }
}

// Candidate quad columns [q_lo, q_hi] of quad row `qy`: the union of the
// candidate tile columns of its (one or two) tile rows inside [y_lo, y_hi).
__device__ __forceinline__ bool band_quads(const Band& e, int qy, int by, int bx, int x_lo, int x_hi, int y_lo,
                                           int y_hi, int& q_lo, int& q_hi)
{
    int lo = 0x7FFFFFFF, hi = -1;
#pragma unroll
    for (int s = 0; s < 2; s++) {
        const int ty = 2 * qy + s;
        int clo = 0, chi = -1;
        if (ty >= y_lo && ty < y_hi && band_columns(e, ty, by, bx, x_lo, x_hi, clo, chi)) {
            lo = min(lo, clo);
            hi = max(hi, chi);
        }
    }
    q_lo = lo >> 1;
    q_hi = hi >> 1;
    return hi >= lo;
}

// sweep_cta over quads: on_step(v, qx, qy, mask) with mask = quad_mask() of
// the quad and v = mask != 0.  A tile that passes the exact test lies in its
// row's band, so its quad lies in the quad row's band.
template <typename F>
__device__ __forceinline__ void sweep_cta_quad(const MassiveEntry& me, const PreprocessParams& a, short2* s_band,
                                               int* s_pref, int* s_wsum, unsigned lane, int warp, F&& on_step)
{
    const float2 c = {me.ctr_power_depth.x, me.ctr_power_depth.y};
    const float pw = me.ctr_power_depth.z;
    const float3 q = {me.conic_gid.x, me.conic_gid.y, me.conic_gid.z};
    const int x_lo = me.rect.x & 0xFFFF, x_hi = me.rect.y, y_lo = me.rect.z, y_hi = me.rect.w;
    const int2 rmin = make_int2(x_lo, y_lo), rmax = make_int2(x_hi, y_hi);
    const int qx_lo = quad_lo(x_lo), qx_hi = quad_hi(x_hi), qy_lo = quad_lo(y_lo), qy_hi = quad_hi(y_hi);
    const Band eb = make_band(q, pw, c);
    if (eb.ok && (qy_hi - qy_lo) <= kMaxBandRows) {
        for (int r = threadIdx.x; r < qy_hi - qy_lo; r += kThreads) {
            int lo = 0, hi = -1;
            if (!band_quads(eb, qy_lo + r, a.by, a.bx, x_lo, x_hi, y_lo, y_hi, lo, hi)) {
                lo = 0;
                hi = -1;
            }
            s_band[r] = make_short2((short)lo, (short)hi);
        }
        __syncthreads();
        sweep_flat_cta(qy_hi - qy_lo, s_band, s_pref, s_wsum, lane, warp, [&](bool valid, int qx, int r) {
            const uint32_t m = valid ? quad_mask(qx, qy_lo + r, rmin, rmax, a.bx, a.by, c, q, pw) : 0u;
            on_step(m != 0u, qx, qy_lo + r, m);
        });
        __syncthreads();
        return;
    }
    // windows of (cols x rows) quads, as sweep_cta does for tiles
    const int w = qx_hi - qx_lo;
    int lg = 5;
    while (lg > 0 && (1 << (lg - 1)) >= w) lg--;
    const int cols = 1 << lg;
    const int rows_w = 32 >> lg;
    const int rows_cta = rows_w * kWarps;
    const int lx = (int)lane & (cols - 1);
    const int ly = warp * rows_w + ((int)lane >> lg);
    for (int wy = qy_lo; wy < qy_hi; wy += rows_cta) {
        const int qy = wy + ly;
        for (int wx = qx_lo; wx < qx_hi; wx += cols) {
            const int qx = wx + lx;
            const uint32_t m =
                (qy < qy_hi && qx < qx_hi) ? quad_mask(qx, qy, rmin, rmax, a.bx, a.by, c, q, pw) : 0u;
            on_step(m != 0u, qx, qy, m);
        }
    }
    __syncthreads();
}

// sweep_warp over quads (see sweep_cta_quad).
template <typename F>
__device__ __forceinline__ void sweep_warp_quad(const MassiveEntry& me, const PreprocessParams& a, unsigned lane,
                                                F&& on_step)
{
    const float2 c = {me.ctr_power_depth.x, me.ctr_power_depth.y};
    const float pw = me.ctr_power_depth.z;
    const float3 q = {me.conic_gid.x, me.conic_gid.y, me.conic_gid.z};
    const int x_lo = me.rect.x & 0xFFFF, x_hi = me.rect.y, y_lo = me.rect.z, y_hi = me.rect.w;
    const int2 rmin = make_int2(x_lo, y_lo), rmax = make_int2(x_hi, y_hi);
    const int qx_lo = quad_lo(x_lo), qx_hi = quad_hi(x_hi), qy_lo = quad_lo(y_lo), qy_hi = quad_hi(y_hi);
    const Band eb = make_band(q, pw, c);
    if (eb.ok) {
        for (int r0 = qy_lo; r0 < qy_hi; r0 += 32) {
            const int qy = r0 + (int)lane;
            int clo = 0, n = 0;
            if (qy < qy_hi) {
                int chi = -1;
                if (band_quads(eb, qy, a.by, a.bx, x_lo, x_hi, y_lo, y_hi, clo, chi)) n = chi - clo + 1;
            }
            int pref = n;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int t = __shfl_up_sync(GSR_FULL_MASK, pref, d);
                if ((int)lane >= d) pref += t;
            }
            const int total = __shfl_sync(GSR_FULL_MASK, pref, 31);
            for (int base = 0; base < total; base += 32) {
                const int task = base + (int)lane;
                int lo = 0, hi = 31;
#pragma unroll
                for (int step = 0; step < 5; step++) {
                    const int mid = (lo + hi) >> 1;
                    if (__shfl_sync(GSR_FULL_MASK, pref, mid) > task) hi = mid;
                    else lo = mid + 1;
                }
                const int o_pref = __shfl_sync(GSR_FULL_MASK, pref, lo);
                const int o_n = __shfl_sync(GSR_FULL_MASK, n, lo);
                const int o_clo = __shfl_sync(GSR_FULL_MASK, clo, lo);
                const int qx = o_clo + task - (o_pref - o_n);
                const int qyy = r0 + lo;
                const uint32_t m = task < total ? quad_mask(qx, qyy, rmin, rmax, a.bx, a.by, c, q, pw) : 0u;
                on_step(m != 0u, qx, qyy, m);
            }
        }
        return;
    }
    const int w = qx_hi - qx_lo;
    const long long total = (long long)w * (long long)(qy_hi - qy_lo);
    for (long long base = 0; base < total; base += 32) {
        const long long t = base + lane;
        int qx = 0, qy = 0;
        uint32_t m = 0u;
        if (t < total) {
            const int r = (int)(t / w);
            qy = qy_lo + r;
            qx = qx_lo + (int)(t - (long long)r * w);
            m = quad_mask(qx, qy, rmin, rmax, a.bx, a.by, c, q, pw);
        }
        on_step(m != 0u, qx, qy, m);
    }
}

// Where the depth-first pipeline's emission pass writes a queued Gaussian.
struct DfEmit {
    const uint32_t* offsets;  // [V] first output position of the s-th Gaussian in depth order
    const uint32_t* rank;     // [P] depth-order position of Gaussian g
    uint32_t* tiles;          // [cap] tile ids, depth-ordered per Gaussian
    uint32_t* vals;           // [cap] Gaussian ids
    long long cap;
};

enum : int { kMassiveEmit64 = 0, kMassiveCount = 1, kMassiveEmitDf = 2 };

// Queued Gaussians: persistent CTAs first take the huge rectangles one at a
// time with all 256 threads, then each warp takes large rectangles on its
// own.  MODE: emit 64-bit keys, count the hit tiles (depth-first counting
// pass), or write depth-first pairs at the Gaussian's offset.
//
// QUAD: the sweeps run over quads (sweep_cta_quad / sweep_warp_quad); a quad
// whose mask is not empty counts as one, and is written as (quad id, index |
// mask << kQuadShift).
template <int MODE, bool VIEWS, bool QUAD = false>
__global__ __launch_bounds__(kThreads) void k_emit_massive(const __grid_constant__ PreprocessParams a, const DfEmit df)
{
    __shared__ uint64_t s_keys[MODE == kMassiveEmit64 ? kWarps : 1][kStage];
    __shared__ uint32_t s_vals[MODE == kMassiveEmit64 ? kWarps : 1][kStage];
    __shared__ int s_fill[kWarps];
    __shared__ long long s_base[kWarps];
    __shared__ int s_entry;
    __shared__ uint32_t s_pos;
    __shared__ uint32_t s_wcnt[kWarps];
    __shared__ short2 s_band[kMaxBandRows];
    __shared__ int s_pref[kMaxBandRows];
    __shared__ int s_wsum[kWarps];
    const unsigned lane = threadIdx.x & 31u;
    const int warp = threadIdx.x >> 5;
    Stage st{s_keys[MODE == kMassiveEmit64 ? warp : 0], s_vals[MODE == kMassiveEmit64 ? warp : 0], 0};
    const EmitOut out{a.keys, a.vals, a.cap, a.counter};
    uint32_t* head = a.mq.head + (MODE == kMassiveEmitDf ? 2 : 0);
    const int n_huge = (int)min(a.mq.count[0], (uint32_t)a.mq.huge_capacity);
    const int n_large = (int)min(a.mq.count[1], (uint32_t)(a.mq.capacity - a.mq.huge_capacity));

    // (1) huge rectangles, one CTA each
    for (;;) {
        if (threadIdx.x == 0) {
            s_entry = (int)atomicAdd(&head[0], 1u);
            s_pos = 0u;
        }
        __syncthreads();
        const int e = s_entry;
        __syncthreads();
        if (e >= n_huge) break;
        const MassiveEntry me = a.mq.entries[e];
        const uint32_t db = __float_as_uint(me.ctr_power_depth.w);
        const uint32_t gid = __float_as_uint(me.conic_gid.w);
        if (VIEWS && ((uint32_t)me.rect.x >> 16) >= (uint32_t)a.n_views) continue;
        const PreprocessParams& av = VIEWS ? a.views[(uint32_t)me.rect.x >> 16] : a;
        if (MODE == kMassiveEmit64 && QUAD) {
            const int qgx = quad_cols(av.gx);
            sweep_cta_quad(me, av, s_band, s_pref, s_wsum, lane, warp, [&](bool v, int qx, int qy, uint32_t m) {
                uint64_t key = ((uint64_t)(uint32_t)(av.tile_base + qy * qgx + qx) << 32) | db;
                stage_emit(st, out, v, key, gid | (m << kQuadShift), lane);
            });
        } else if (MODE == kMassiveEmit64) {
            sweep_cta(me, av, s_band, s_pref, s_wsum, lane, warp, [&](bool v, int x, int y) {
                uint64_t key = ((uint64_t)(uint32_t)(av.tile_base + y * av.gx + x) << 32) | db;
                stage_emit(st, out, v, key, gid, lane);
            });
        } else if (MODE == kMassiveCount) {
            uint32_t cnt = 0;
            if (QUAD)
                sweep_cta_quad(me, a, s_band, s_pref, s_wsum, lane, warp, [&](bool v, int, int, uint32_t) {
                    cnt += __popc(__ballot_sync(GSR_FULL_MASK, v));
                });
            else
                sweep_cta(me, a, s_band, s_pref, s_wsum, lane, warp, [&](bool v, int, int) {
                    cnt += __popc(__ballot_sync(GSR_FULL_MASK, v));
                });
            if (lane == 0) s_wcnt[warp] = cnt;
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t t = 0;
                for (int w = 0; w < kWarps; w++) t += s_wcnt[w];
                a.df.count[gid] = t;
            }
        } else {
            // Gaussians that hit no tile were not ranked
            const uint32_t count = a.df.count[gid];
            if (count == 0u) continue;
            const long long base = df.offsets[df.rank[gid]];
            // a pair (tile id, value) at the next of the Gaussian's own slots
            auto put = [&](bool v, uint32_t tile, uint32_t val) {
                const unsigned m = __ballot_sync(GSR_FULL_MASK, v);
                if (!m) return;
                uint32_t w0 = 0;
                if (lane == 0) w0 = atomicAdd(&s_pos, (uint32_t)__popc(m));
                w0 = __shfl_sync(GSR_FULL_MASK, w0, 0);
                const uint32_t k = w0 + __popc(m & lanemask_lt());
                if (v && k < count && base + k < df.cap) {  // never past the Gaussian's own slots
                    df.tiles[base + k] = tile;
                    df.vals[base + k] = val;
                }
            };
            if (QUAD) {
                const int qgx = quad_cols(a.gx);
                sweep_cta_quad(me, a, s_band, s_pref, s_wsum, lane, warp, [&](bool v, int qx, int qy, uint32_t m) {
                    put(v, (uint32_t)(qy * qgx + qx), gid | (m << kQuadShift));
                });
            } else {
                sweep_cta(me, a, s_band, s_pref, s_wsum, lane, warp,
                          [&](bool v, int x, int y) { put(v, (uint32_t)(y * a.gx + x), gid); });
            }
            // sweep_cta ended on a barrier, so s_pos is final; every thread
            // reads it before thread 0 resets it for the next entry
            const uint32_t filled = s_pos;
            __syncthreads();
            for (uint32_t k = filled + threadIdx.x; k < count; k += kThreads)  // pad unfilled slots
                if (base + k < df.cap) {
                    df.tiles[base + k] = kTileSentinel;
                    df.vals[base + k] = kTileSentinel;
                }
        }
    }

    // (2) large rectangles, one warp each
    for (;;) {
        int e = 0;
        if (lane == 0) e = (int)atomicAdd(&head[1], 1u);
        e = __shfl_sync(GSR_FULL_MASK, e, 0);
        if (e >= n_large) break;
        const MassiveEntry me = a.mq.entries[a.mq.huge_capacity + e];
        const uint32_t db = __float_as_uint(me.ctr_power_depth.w);
        const uint32_t gid = __float_as_uint(me.conic_gid.w);
        if (VIEWS && ((uint32_t)me.rect.x >> 16) >= (uint32_t)a.n_views) continue;
        const PreprocessParams& av = VIEWS ? a.views[(uint32_t)me.rect.x >> 16] : a;
        if (MODE == kMassiveEmit64 && QUAD) {
            const int qgx = quad_cols(av.gx);
            sweep_warp_quad(me, av, lane, [&](bool v, int qx, int qy, uint32_t m) {
                uint64_t key = ((uint64_t)(uint32_t)(av.tile_base + qy * qgx + qx) << 32) | db;
                stage_emit(st, out, v, key, gid | (m << kQuadShift), lane);
            });
        } else if (MODE == kMassiveEmit64) {
            sweep_warp(me, av, lane, [&](bool v, int x, int y) {
                uint64_t key = ((uint64_t)(uint32_t)(av.tile_base + y * av.gx + x) << 32) | db;
                stage_emit(st, out, v, key, gid, lane);
            });
        } else if (MODE == kMassiveCount) {
            uint32_t cnt = 0;
            if (QUAD)
                sweep_warp_quad(me, a, lane,
                                [&](bool v, int, int, uint32_t) { cnt += __popc(__ballot_sync(GSR_FULL_MASK, v)); });
            else
                sweep_warp(me, a, lane, [&](bool v, int, int) { cnt += __popc(__ballot_sync(GSR_FULL_MASK, v)); });
            if (lane == 0) a.df.count[gid] = cnt;
        } else {
            const uint32_t count = a.df.count[gid];
            if (count == 0u) continue;
            const long long base = df.offsets[df.rank[gid]];
            uint32_t wpos = 0;
            auto put = [&](bool v, uint32_t tile, uint32_t val) {
                const unsigned m = __ballot_sync(GSR_FULL_MASK, v);
                const uint32_t k = wpos + __popc(m & lanemask_lt());
                if (v && k < count && base + k < df.cap) {
                    df.tiles[base + k] = tile;
                    df.vals[base + k] = val;
                }
                wpos += __popc(m);
            };
            if (QUAD) {
                const int qgx = quad_cols(a.gx);
                sweep_warp_quad(me, a, lane, [&](bool v, int qx, int qy, uint32_t m) {
                    put(v, (uint32_t)(qy * qgx + qx), gid | (m << kQuadShift));
                });
            } else {
                sweep_warp(me, a, lane, [&](bool v, int x, int y) { put(v, (uint32_t)(y * a.gx + x), gid); });
            }
            for (uint32_t k = wpos + lane; k < count; k += 32)
                if (base + k < df.cap) {
                    df.tiles[base + k] = kTileSentinel;
                    df.vals[base + k] = kTileSentinel;
                }
        }
    }
    if (MODE == kMassiveEmit64) block_flush(st, out, s_fill, s_base, lane, warp);
}

// Depth-first emission of the Gaussians that were not queued, taken in depth
// order: each writes its (tile, index) pairs from its offset on.  Each warp
// takes 32 consecutive Gaussians of the order; a rectangle under
// massive_area tiles is swept by its own thread, a larger one (a Gaussian
// the full large-Gaussian queue turned away) by the whole warp in 8 x 4
// windows, as the counting pass swept it.  Same tile test as the counting
// pass, so exactly count[g] pairs; slots a Gaussian cannot fill are padded.
//
// QUAD: the Gaussian's quads, each with a non-empty mask, as (quad id, index |
// mask << kQuadShift).
template <bool QUAD>
__global__ __launch_bounds__(256, 2) void k_df_emit_small(const PreprocessParams a, const DfEmit df,
                                                       const uint32_t* __restrict__ d_v,
                                                       const uint32_t* __restrict__ sgids)
{
    const int V = (int)min(*d_v, (uint32_t)a.P);
    const unsigned lane = threadIdx.x & 31u;
    const int qgx = quad_cols(a.gx);
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long s0 = ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; s0 < V;
         s0 += warps * 32) {
        const long long s = s0 + lane;
        uint32_t gid = 0u, count = 0u;
        int x0 = 0, x1 = 0, y0 = 0, y1 = 0;
        long long pos = 0;
        bool own = false, wide = false;
        if (s < V) {
            gid = __ldg(sgids + s);
            if (gid < (uint32_t)a.P) {
                const int2 r = __ldg(a.df.rect + gid);
                if (!((uint32_t)r.y & 0x80000000u)) {  // queued ones: the massive kernel writes them
                    x0 = r.x & 0xFFFF;
                    x1 = (int)((uint32_t)r.x >> 16);
                    y0 = r.y & 0xFFFF;
                    y1 = (int)(((uint32_t)r.y >> 16) & 0x7FFFu);
                    pos = __ldg(df.offsets + s);
                    count = __ldg(a.df.count + gid);
                    wide = (x1 - x0) * (y1 - y0) >= a.massive_area;
                    own = !wide;
                }
            }
        }
        const float4 g = own || wide ? __ldg(a.df.geo + gid) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float2 ctr = own || wide ? __ldg(a.points_xy + gid) : make_float2(0.f, 0.f);
        if (own) {
            const float3 con = {g.x, g.y, g.z};
            const long long lim = pos + count;  // the Gaussian's own slots
            if (QUAD) {
                for (int qy = quad_lo(y0); qy < quad_hi(y1); qy++)
                    for (int qx = quad_lo(x0); qx < quad_hi(x1); qx++) {
                        const uint32_t m =
                            quad_mask(qx, qy, make_int2(x0, y0), make_int2(x1, y1), a.bx, a.by, ctr, con, g.w);
                        if (!m) continue;
                        if (pos < lim && pos < df.cap) {
                            df.tiles[pos] = (uint32_t)(qy * qgx + qx);
                            df.vals[pos] = gid | (m << kQuadShift);
                        }
                        pos++;
                    }
            } else {
                for (int y = y0; y < y1; y++)
                    for (int x = x0; x < x1; x++) {
                        if (!tile_hit(x, y, a.bx, a.by, ctr, con, g.w)) continue;
                        if (pos < lim && pos < df.cap) {
                            df.tiles[pos] = (uint32_t)(y * a.gx + x);
                            df.vals[pos] = gid;
                        }
                        pos++;
                    }
            }
            for (; pos < lim; pos++)  // pad unfilled slots
                if (pos < df.cap) {
                    df.tiles[pos] = kTileSentinel;
                    df.vals[pos] = kTileSentinel;
                }
        }
        // the wide rectangles, one after another, by the whole warp
        unsigned todo = __ballot_sync(GSR_FULL_MASK, wide);
        while (todo) {
            const int i = __ffs(todo) - 1;
            todo &= todo - 1;
            const uint32_t wg = __shfl_sync(GSR_FULL_MASK, gid, i);
            const uint32_t wcount = __shfl_sync(GSR_FULL_MASK, count, i);
            const long long base = __shfl_sync(GSR_FULL_MASK, pos, i);
            const int2 rmin = make_int2(__shfl_sync(GSR_FULL_MASK, x0, i), __shfl_sync(GSR_FULL_MASK, y0, i));
            const int2 rmax = make_int2(__shfl_sync(GSR_FULL_MASK, x1, i), __shfl_sync(GSR_FULL_MASK, y1, i));
            const float2 c = {__shfl_sync(GSR_FULL_MASK, ctr.x, i), __shfl_sync(GSR_FULL_MASK, ctr.y, i)};
            const float3 q = {__shfl_sync(GSR_FULL_MASK, g.x, i), __shfl_sync(GSR_FULL_MASK, g.y, i),
                              __shfl_sync(GSR_FULL_MASK, g.z, i)};
            const float pw = __shfl_sync(GSR_FULL_MASK, g.w, i);
            uint32_t wpos = 0;
            auto put = [&](bool v, uint32_t tile, uint32_t val) {
                const unsigned m = __ballot_sync(GSR_FULL_MASK, v);
                const uint32_t k = wpos + __popc(m & lanemask_lt());
                if (v && k < wcount && base + k < df.cap) {
                    df.tiles[base + k] = tile;
                    df.vals[base + k] = val;
                }
                wpos += __popc(m);
            };
            const int tx = (int)(lane & 7u), ty = (int)(lane >> 3);
            if (QUAD) {
                const int qx_lo = quad_lo(rmin.x), qx_hi = quad_hi(rmax.x);
                const int qy_lo = quad_lo(rmin.y), qy_hi = quad_hi(rmax.y);
                for (int yy = qy_lo; yy < qy_hi; yy += 4)
                    for (int xx = qx_lo; xx < qx_hi; xx += 8) {
                        const int qx = xx + tx, qy = yy + ty;
                        const uint32_t m = (qx < qx_hi && qy < qy_hi)
                                               ? quad_mask(qx, qy, rmin, rmax, a.bx, a.by, c, q, pw)
                                               : 0u;
                        put(m != 0u, (uint32_t)(qy * qgx + qx), wg | (m << kQuadShift));
                    }
            } else {
                for (int yy = rmin.y; yy < rmax.y; yy += 4)
                    for (int xx = rmin.x; xx < rmax.x; xx += 8) {
                        const int x = xx + tx, y = yy + ty;
                        const bool v = x < rmax.x && y < rmax.y && tile_hit(x, y, a.bx, a.by, c, q, pw);
                        put(v, (uint32_t)(y * a.gx + x), wg);
                    }
            }
            for (uint32_t k = wpos + lane; k < wcount; k += 32)  // pad unfilled slots
                if (base + k < df.cap) {
                    df.tiles[base + k] = kTileSentinel;
                    df.vals[base + k] = kTileSentinel;
                }
        }
    }
}

// ---------------------------------------------------------------------------
// Scene preparation (pybind.cpp:22-56, 105-117) on the device.
__global__ void k_scene_prepare(int P, const float* __restrict__ log_scales, const float* __restrict__ quats,
                                const float* __restrict__ logits, float* __restrict__ opacity,
                                float* __restrict__ cov3d)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    opacity[i] = 1.0f / (1.0f + expf(-logits[i]));
    float sx = expf(log_scales[3 * i]), sy = expf(log_scales[3 * i + 1]), sz = expf(log_scales[3 * i + 2]);
    float4 q = reinterpret_cast<const float4*>(quats)[i];
    float inv = rsqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    float r = q.x * inv, x = q.y * inv, y = q.z * inv, z = q.w * inv;
    M3 S = m3_cols(sx, 0.f, 0.f, 0.f, sy, 0.f, 0.f, 0.f, sz);
    M3 R = m3_cols(1.f - 2.f * (y * y + z * z), 2.f * (x * y - r * z), 2.f * (x * z + r * y),
                   2.f * (x * y + r * z), 1.f - 2.f * (x * x + z * z), 2.f * (y * z - r * x),
                   2.f * (x * z - r * y), 2.f * (y * z + r * x), 1.f - 2.f * (x * x + y * y));
    M3 M = m3_mul(S, R);
    M3 Sg = m3_mul(m3_transpose(M), M);
    float* c = cov3d + 6 * (size_t)i;
    c[0] = Sg.m[0][0];
    c[1] = Sg.m[0][1];
    c[2] = Sg.m[0][2];
    c[3] = Sg.m[1][1];
    c[4] = Sg.m[1][2];
    c[5] = Sg.m[2][2];
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side: view / projection matrices (preprocess.cu:643-671), column-major.

static void mat4_mul(const float* a, const float* b, float* r)  // r = a * b, column-major
{
    for (int c = 0; c < 4; c++)
        for (int k = 0; k < 4; k++)
            r[4 * c + k] = a[0 * 4 + k] * b[4 * c + 0] + a[1 * 4 + k] * b[4 * c + 1] + a[2 * 4 + k] * b[4 * c + 2] +
                           a[3 * 4 + k] * b[4 * c + 3];
}

void camera_matrices(int W, int H, const float* pos, const float* rot, float fx, float fy, float zfar, float znear,
                     float* view, float* proj)
{
    // glm::mat3 built from the rows of `rot`: column c = rot row c.
    float R[3][3];
    for (int c = 0; c < 3; c++)
        for (int k = 0; k < 3; k++) R[c][k] = rot[3 * c + k];
    float np[3] = {-pos[0], -pos[1], -pos[2]};
    float t[3];
    for (int k = 0; k < 3; k++) t[k] = R[0][k] * np[0] + R[1][k] * np[1] + R[2][k] * np[2];
    for (int c = 0; c < 3; c++) {
        for (int k = 0; k < 3; k++) view[4 * c + k] = R[c][k];
        view[4 * c + 3] = 0.0f;
    }
    view[12] = t[0];
    view[13] = t[1];
    view[14] = t[2];
    view[15] = 1.0f;

    float top = H / (2.0f * fy) * znear;
    float bottom = -top;
    float right = W / (2.0f * fx) * znear;
    float left = -right;
    float P[16];
    for (int i = 0; i < 16; i++) P[i] = 0.0f;
    const float z_sign = 1.0f;
    P[0 * 4 + 0] = 2.0f * znear / (right - left);
    P[1 * 4 + 1] = 2.0f * znear / (top - bottom);
    P[0 * 4 + 2] = (right + left) / (right - left);
    P[1 * 4 + 2] = (top + bottom) / (top - bottom);
    P[3 * 4 + 2] = z_sign;
    P[2 * 4 + 2] = z_sign * zfar / (zfar - znear);
    P[2 * 4 + 3] = -(zfar * znear) / (zfar - znear);
    float PT[16];
    for (int c = 0; c < 4; c++)
        for (int k = 0; k < 4; k++) PT[4 * c + k] = P[4 * k + c];
    mat4_mul(PT, view, proj);
}

cudaError_t launch_scene_prepare(int P, const float* log_scales, const float* quats, const float* logits,
                                 float* opacity, float* cov3d, cudaStream_t stream)
{
    if (P <= 0) return cudaSuccess;
    k_scene_prepare<<<div_up(P, 256), 256, 0, stream>>>(P, log_scales, quats, logits, opacity, cov3d);
    return cudaGetLastError();
}

// Persistent grid of the queue sweeps: as many CTAs as fit on every SM.
template <typename Kern>
static int emit_grid(Kern kern)
{
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, kThreads, 0) != cudaSuccess || b < 1) b = 4;
    return device_sm_count() * b;
}

static cudaError_t preprocess_common(const PreprocessParams& p, bool half_sh, bool count, cudaStream_t stream)
{
    if (p.P <= 0) return cudaSuccess;
    if (p.mq.capacity > 0) {
        // queue counters, heads of both passes and depth_hi: the preprocess
        // region of the workspace header, which starts at the count words
        cudaError_t e = cudaMemsetAsync(p.mq.count, 0, kPreprocessRegionBytes, stream);
        if (e != cudaSuccess) return e;
    }
    if (p.quad && (p.bx != 16 || p.by != 16 || p.df.ref_layout)) return cudaErrorInvalidValue;
    const int grid = div_up(p.P, kThreads);
    if (count && p.quad) {
        if (half_sh) k_preprocess<true, true, false, true><<<grid, kThreads, 0, stream>>>(p);
        else k_preprocess<false, true, false, true><<<grid, kThreads, 0, stream>>>(p);
    } else if (count) {
        if (half_sh) k_preprocess<true, true, false><<<grid, kThreads, 0, stream>>>(p);
        else k_preprocess<false, true, false><<<grid, kThreads, 0, stream>>>(p);
    } else if (p.quad) {
        if (half_sh) k_preprocess<true, false, false, true><<<grid, kThreads, 0, stream>>>(p);
        else k_preprocess<false, false, false, true><<<grid, kThreads, 0, stream>>>(p);
    } else {
        if (half_sh) k_preprocess<true, false, false><<<grid, kThreads, 0, stream>>>(p);
        else k_preprocess<false, false, false><<<grid, kThreads, 0, stream>>>(p);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || p.mq.capacity <= 0) return e;
    const DfEmit none{nullptr, nullptr, nullptr, nullptr, 0};
    if (count && p.quad)
        k_emit_massive<kMassiveCount, false, true>
            <<<emit_grid(k_emit_massive<kMassiveCount, false, true>), kThreads, 0, stream>>>(p, none);
    else if (count) k_emit_massive<kMassiveCount, false><<<emit_grid(k_emit_massive<kMassiveCount, false>), kThreads, 0, stream>>>(p, none);
    else if (p.quad)
        k_emit_massive<kMassiveEmit64, false, true>
            <<<emit_grid(k_emit_massive<kMassiveEmit64, false, true>), kThreads, 0, stream>>>(p, none);
    else k_emit_massive<kMassiveEmit64, false><<<emit_grid(k_emit_massive<kMassiveEmit64, false>), kThreads, 0, stream>>>(p, none);
    return cudaGetLastError();
}

cudaError_t launch_preprocess_views(const PreprocessParams& base, int n_views, int blocks, bool half_sh,
                                    cudaStream_t stream)
{
    if (n_views <= 0 || blocks <= 0) return cudaSuccess;
    if (n_views > 32767 || !base.views || base.mq.capacity <= 0) return cudaErrorInvalidValue;
    if (base.quad && (base.bx != 16 || base.by != 16)) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(base.mq.count, 0, kPreprocessRegionBytes, stream);
    if (e != cudaSuccess) return e;
    const dim3 grid(blocks);
    const DfEmit none{nullptr, nullptr, nullptr, nullptr, 0};
    if (base.quad) {
        // every view's block carries the same quad flag as the base block
        if (half_sh) k_preprocess<true, false, true, true><<<grid, kThreads, 0, stream>>>(base);
        else k_preprocess<false, false, true, true><<<grid, kThreads, 0, stream>>>(base);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        k_emit_massive<kMassiveEmit64, true, true>
            <<<emit_grid(k_emit_massive<kMassiveEmit64, true, true>), kThreads, 0, stream>>>(base, none);
        return cudaGetLastError();
    }
    if (half_sh) k_preprocess<true, false, true><<<grid, kThreads, 0, stream>>>(base);
    else k_preprocess<false, false, true><<<grid, kThreads, 0, stream>>>(base);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_emit_massive<kMassiveEmit64, true><<<emit_grid(k_emit_massive<kMassiveEmit64, true>), kThreads, 0, stream>>>(base, none);
    return cudaGetLastError();
}

cudaError_t launch_preprocess(const PreprocessParams& p, bool half_sh, cudaStream_t stream)
{
    return preprocess_common(p, half_sh, false, stream);
}

cudaError_t launch_preprocess_count(const PreprocessParams& p, bool half_sh, cudaStream_t stream)
{
    return preprocess_common(p, half_sh, true, stream);
}

cudaError_t launch_df_emit_massive(const PreprocessParams& p, const uint32_t* offsets, const uint32_t* rank,
                                   uint32_t* tiles, uint32_t* vals, long long cap, cudaStream_t stream)
{
    if (p.P <= 0 || p.mq.capacity <= 0) return cudaSuccess;
    // takes the queue again through the second pair of heads (cleared with
    // the rest of the preprocess region before the counting pass)
    const DfEmit df{offsets, rank, tiles, vals, cap};
    if (p.quad)
        k_emit_massive<kMassiveEmitDf, false, true>
            <<<emit_grid(k_emit_massive<kMassiveEmitDf, false, true>), kThreads, 0, stream>>>(p, df);
    else
        k_emit_massive<kMassiveEmitDf, false>
            <<<emit_grid(k_emit_massive<kMassiveEmitDf, false>), kThreads, 0, stream>>>(p, df);
    return cudaGetLastError();
}

// The reference's ES pass B (preprocess.cu:993-1248): every Gaussian in
// depth order writes its (tile id, index) pairs from its scanned offset on,
// from the counting pass's records alone (centre, raw conic + power, packed
// rectangle).  One warp per Gaussian sweeps its candidate tiles with the
// counting pass's tile test, so it writes exactly the counted pairs.
__global__ __launch_bounds__(256) void k_es_pass_b(int P, int bx, int by, int gx, const uint32_t* __restrict__ perm,
                                                   const int32_t* __restrict__ cum,
                                                   const int32_t* __restrict__ count_sorted,
                                                   const float2* __restrict__ xy, const float4* __restrict__ cpr,
                                                   const int2* __restrict__ rb, uint32_t* __restrict__ tiles,
                                                   uint32_t* __restrict__ vals, long long cap)
{
    const unsigned lane = threadIdx.x & 31u;
    PreprocessParams pp;
    pp.bx = bx;
    pp.by = by;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long s = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); s < P; s += warps) {
        const int c = __ldg(count_sorted + s);
        if (c <= 0) continue;
        const uint32_t gid = __ldg(perm + s);
        if (gid >= (uint32_t)P) continue;
        const long long base = __ldg(cum + s);
        const float2 ctr = __ldg(xy + gid);
        const float4 cp = __ldg(cpr + gid);
        const int2 r = __ldg(rb + gid);
        MassiveEntry me;
        me.ctr_power_depth = make_float4(ctr.x, ctr.y, cp.w, 0.f);
        me.conic_gid = make_float4(cp.x, cp.y, cp.z, __uint_as_float(gid));
        // rect_min / rect_max unpacked as signed 16-bit (preprocess.cu:1043-1048); clamped to the grid
        const int x0 = max(0, (int)(int16_t)(r.x & 0xFFFF)), y0 = max(0, (int)(int16_t)((r.x >> 16) & 0xFFFF));
        const int x1 = min(gx, (int)(int16_t)(r.y & 0xFFFF)), y1 = (int)(int16_t)((r.y >> 16) & 0xFFFF);
        me.rect = make_int4(x0, max(x0, x1), y0, max(y0, y1));
        uint32_t wpos = 0;
        sweep_warp(me, pp, lane, [&](bool v, int x, int y) {
            const unsigned m = __ballot_sync(GSR_FULL_MASK, v);
            if (v) {
                const long long pos = base + wpos + __popc(m & lanemask_lt());
                if (pos >= 0 && pos < cap && wpos + __popc(m & lanemask_lt()) < (uint32_t)c) {
                    tiles[pos] = (uint32_t)(y * gx + x);
                    vals[pos] = gid;
                }
            }
            wpos += __popc(m);
        });
        for (uint32_t k = wpos + lane; k < (uint32_t)c; k += 32)  // pad unfilled slots
            if (base + k >= 0 && base + k < cap) {
                tiles[base + k] = kTileSentinel;
                vals[base + k] = kTileSentinel;
            }
    }
}

cudaError_t launch_es_pass_b(int P, int bx, int by, int gx, const uint32_t* perm, const int32_t* cum,
                             const int32_t* count_sorted, const float2* xy, const float4* cpr, const int2* rb,
                             uint32_t* tiles, uint32_t* vals, long long cap, cudaStream_t stream)
{
    if (P <= 0) return cudaSuccess;
    const int grid = std::min(div_up(P, 8), device_sm_count() * 8);
    k_es_pass_b<<<grid, 256, 0, stream>>>(P, bx, by, gx, perm, cum, count_sorted, xy, cpr, rb, tiles, vals, cap);
    return cudaGetLastError();
}

cudaError_t launch_df_emit_small(const PreprocessParams& p, const uint32_t* d_v, const uint32_t* sgids,
                                 const uint32_t* offsets, uint32_t* tiles, uint32_t* vals, long long cap,
                                 cudaStream_t stream)
{
    if (p.P <= 0) return cudaSuccess;
    const DfEmit df{offsets, nullptr, tiles, vals, cap};
    const int grid = std::min(div_up(p.P, 256), device_sm_count() * 8);
    if (p.quad) k_df_emit_small<true><<<grid, 256, 0, stream>>>(p, df, d_v, sgids);
    else k_df_emit_small<false><<<grid, 256, 0, stream>>>(p, df, d_v, sgids);
    return cudaGetLastError();
}

}  // namespace gsr
