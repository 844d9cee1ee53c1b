// Persistent tile-queue blend for sm_103a.
//
// One warp renders one tile at a time; every lane owns a (BX/8) x (BY/4)
// block of pixels (8 x 4 lanes over the tile, csrc/cuda_rasterizer/
// render.cu:1736-1737).  Warps take tiles from a per-launch atomic queue in
// the caller's workspace (no module-global counter, so concurrent launches on
// different workspaces are safe).  The Gaussians of a tile are consumed in
// batches of 32: for each batch every lane copies its Gaussian's
// conic/opacity, colour/depth and centre records into one half of a
// double-buffered shared-memory ring with per-thread cp.async copies, so the
// next batch streams in while the current one is blended.  A second staging
// path issues 1-D TMA bulk copies (cp.async.bulk) completed on an mbarrier
// (GSR_RENDER_TMA=1); for these 16-byte gathers it measured slower.  Every
// wait is bounded: on expiry the warp records a timeout in the status word
// and stops.
//
// The blend of each Gaussian-pixel pair is the reference's arithmetic
// (pixel_shader_axis_shared_16x16 / pixel_shader, render.cu:228-271 and
// 216-226): alpha = ex2.approx.ftz(power) with no 0.99 clamp and no 1/255
// skip, front-to-back compositing, and a whole-tile exit once every pixel of
// the tile has T < 1e-4, checked every CADENCE Gaussians.  Output is the
// truncating uint8 encode of render.cu:375-394.
#include <atomic>
#include <cstdlib>
#include <cstring>

#include "gsr_internal.h"

namespace gsr {
namespace {

constexpr int kRenderWarps = 4;
constexpr int kBatch = 32;

struct WarpRing {
    float4 con[2][kBatch];
    float4 rgbd[2][kBatch];
    float4 xy2[2][kBatch];  // 16-byte pair holding the Gaussian's centre
    uint32_t sel[2][kBatch];
    uint64_t bar[2];
};

struct RenderParams {
    int n_host;
    const int32_t* d_num;
    long long cap;
    int W, H, gx, tiles, P;  // quad renders: gx and tiles count quads
    int items;               // work items: tiles, or 4 per quad
    const float2* xy;
    const float4* rgbd;
    const float4* con;
    const uint64_t* keys;
    const uint32_t* vals;
    const int2* ranges;
    float3 bg;
    uchar3* out;
    uint32_t* queue;
    uint32_t* status;
    const RenderView* views;  // batched render: per-view blocks (nullptr: one view)
    int n_views;
};

__device__ __forceinline__ uint8_t encode8(float x) { return (uint8_t)fminf(fmaxf(0.0f, x * 255.0f), 255.0f); }

// Final colour of a pixel: C + T' bg with T' = 0 once T < 1e-4; background
// only for a tile without Gaussians (render.cu:375-394, 1845-1858).
__device__ __forceinline__ uchar3 encode_px(const float (&c)[3], float t, bool any, float3 bg)
{
    if (t < 0.0001f) t = 0.0f;
    uchar3 o;
    if (any) {
        o.x = encode8(c[0] + t * bg.x);
        o.y = encode8(c[1] + t * bg.y);
        o.z = encode8(c[2] + t * bg.z);
    } else {
        o.x = encode8(bg.x);
        o.y = encode8(bg.y);
        o.z = encode8(bg.z);
    }
    return o;
}

// First index in keys[lo, hi) whose tile id is > t (UPPER) or >= t (!UPPER);
// warp-cooperative 32-way search, log32(n) rounds.
template <bool UPPER>
__device__ __forceinline__ int warp_bound(const uint64_t* __restrict__ keys, int lo, int hi, uint32_t t, unsigned lane)
{
    while (hi - lo > 32) {
        const int step = (hi - lo + 31) >> 5;
        const int p = lo + ((int)lane + 1) * step - 1;
        bool pred = false;
        if (p < hi) {
            const uint32_t kt = (uint32_t)(__ldg(keys + p) >> 32);
            pred = UPPER ? (kt <= t) : (kt < t);
        }
        const int c = __popc(__ballot_sync(GSR_FULL_MASK, pred));
        const int nlo = c == 0 ? lo : lo + c * step;  // first probe that failed is p_c
        const int nhi = min(hi, lo + (c + 1) * step);
        lo = nlo;
        hi = nhi;
    }
    const int p = lo + (int)lane;
    bool pred = false;
    if (p < hi) {
        const uint32_t kt = (uint32_t)(__ldg(keys + p) >> 32);
        pred = UPPER ? (kt <= t) : (kt < t);
    }
    return lo + __popc(__ballot_sync(GSR_FULL_MASK, pred));
}

// Stage the next Gaussians of the tile's list, from position `pos` on, into
// ring half `b`, and advance `pos` past them; returns how many were staged.
// Per-tile lists: the next min(32, end - pos).  QUAD: the quad's list is
// scanned from `pos` on until 32 values with bit `sub_bit` set (the
// Gaussians of this warp's tile of the quad) are staged, in list order, or
// the list ends -- so a batch is as full as in a per-tile list.
template <bool TMA, bool QUAD = false>
__device__ __forceinline__ int stage_batch(WarpRing& R, int b, const RenderParams& p, int& pos, int end,
                                           unsigned lane, bool& bad, uint32_t sub_bit = 0u)
{
    __syncwarp();
    if (TMA) fence_proxy_async_smem();
    if (QUAD) {
        static_assert(!QUAD || !TMA, "quad renders stage with cp.async");
        int filled = 0;
        while (filled < kBatch && pos < end) {
            const int cnt = min(kBatch, end - pos);
            uint32_t v = 0u;
            if ((int)lane < cnt) v = __ldg(p.vals + pos + lane);
            const bool hit = (int)lane < cnt && (v & sub_bit) != 0u;
            const unsigned hits = __ballot_sync(GSR_FULL_MASK, hit);
            const int room = kBatch - filled;
            const int rank = __popc(hits & lanemask_lt());
            uint32_t gid = v & kQuadGidMask;
            if (hit && rank < room) {
                if (gid < (uint32_t)p.P) {
                    const int slot = filled + rank;
                    cp_async_16(&R.con[b][slot], p.con + gid);
                    cp_async_16(&R.rgbd[b][slot], p.rgbd + gid);
                    cp_async_8(&R.xy2[b][slot], p.xy + gid);
                    R.sel[b][slot] = 0u;
                } else {  // index outside the feature arrays: a transparent stand-in
                    bad = true;
                    const int slot = filled + rank;
                    R.con[b][slot] = make_float4(0.f, 0.f, 0.f, -1e30f);
                    R.rgbd[b][slot] = make_float4(0.f, 0.f, 0.f, 0.f);
                    R.xy2[b][slot] = make_float4(0.f, 0.f, 0.f, 0.f);
                    R.sel[b][slot] = 0u;
                }
            }
            const int n = __popc(hits);
            if (n <= room) {
                pos += cnt;
                filled += n;
            } else {
                // the batch is full: resume right after its last Gaussian
                pos += __ffs(__ballot_sync(GSR_FULL_MASK, hit && rank == room - 1));
                filled = kBatch;
            }
        }
        cp_async_commit();
        return filled;
    }
    const int cnt = min(kBatch, end - pos);
    pos += cnt;
    const int base = pos - cnt;
    uint32_t gid = 0;
    bool ok = (int)lane < cnt;
    if (ok) {
        gid = __ldg(p.vals + base + lane);
        if (gid >= (uint32_t)p.P) {  // index outside the feature arrays: skip it
            ok = false;
            bad = true;
        }
    }
    const bool pair_ok = ok && (gid | 1u) < (uint32_t)p.P;
    if (TMA) {
        const uint32_t tx = 32u * __popc(__ballot_sync(GSR_FULL_MASK, ok)) + 16u * __popc(__ballot_sync(GSR_FULL_MASK, pair_ok));
        if (lane == 0) mbar_arrive_expect_tx(&R.bar[b], tx);
        __syncwarp();
        if (ok) {
            tma_bulk_g2s(&R.con[b][lane], p.con + gid, 16, &R.bar[b]);
            tma_bulk_g2s(&R.rgbd[b][lane], p.rgbd + gid, 16, &R.bar[b]);
            if (pair_ok) {
                tma_bulk_g2s(&R.xy2[b][lane], p.xy + (gid & ~1u), 16, &R.bar[b]);
                R.sel[b][lane] = gid & 1u;
            } else {
                const float2 v = __ldg(p.xy + gid);
                R.xy2[b][lane] = make_float4(v.x, v.y, 0.f, 0.f);
                R.sel[b][lane] = 0u;
            }
        }
        if (!ok && (int)lane < cnt) {  // skipped index: a fully transparent stand-in
            R.con[b][lane] = make_float4(0.f, 0.f, 0.f, -1e30f);
            R.rgbd[b][lane] = make_float4(0.f, 0.f, 0.f, 0.f);
            R.xy2[b][lane] = make_float4(0.f, 0.f, 0.f, 0.f);
            R.sel[b][lane] = 0u;
        }
    } else {
        if (ok) {
            cp_async_16(&R.con[b][lane], p.con + gid);
            cp_async_16(&R.rgbd[b][lane], p.rgbd + gid);
            cp_async_8(&R.xy2[b][lane], p.xy + gid);
            R.sel[b][lane] = 0u;
        } else if ((int)lane < cnt) {
            R.con[b][lane] = make_float4(0.f, 0.f, 0.f, -1e30f);
            R.rgbd[b][lane] = make_float4(0.f, 0.f, 0.f, 0.f);
            R.xy2[b][lane] = make_float4(0.f, 0.f, 0.f, 0.f);
            R.sel[b][lane] = 0u;
        }
        cp_async_commit();
    }
    return cnt;
}

// Wait until ring half `b` is filled.  Returns false on timeout.
template <bool TMA>
__device__ __forceinline__ bool wait_batch(WarpRing& R, int b, uint32_t& phase_bits)
{
    bool ok = true;
    if (TMA) {
        ok = mbar_wait_bounded(&R.bar[b], (phase_bits >> b) & 1u);
        phase_bits ^= 1u << b;
    } else {
        cp_async_wait_all();
    }
    __syncwarp();
    return ok;
}

// SHADER 0: pixel_shader_axis_shared_16x16 (render.cu:228-271)
// SHADER 1: pixel_shader (render.cu:216-226)
template <int TX, int TY, int SHADER, bool DT>
__device__ __forceinline__ void shade(float (&C)[TY][TX][3], float (&T)[TY][TX], int ox, int oy, int cb, int rb,
                                      float2 xy, float4 co, float3 rgb)
{
    if (SHADER == 0) {
        float xs[TX], xc[TX];
#pragma unroll
        for (int j = 0; j < TX; j++) {
            float dx = xy.x - (float)(ox + cb + j);
            xs[j] = co.x * dx * dx;
            xc[j] = co.y * dx;
        }
        float yd[TY], ys[TY];
#pragma unroll
        for (int i = 0; i < TY; i++) {
            float dy = xy.y - (float)(oy + rb + i);
            yd[i] = dy;
            ys[i] = co.z * dy * dy;
        }
#pragma unroll
        for (int i = 0; i < TY; i++)
#pragma unroll
            for (int j = 0; j < TX; j++) {
                float power = fmaf(xc[j], yd[i], co.w + xs[j] + ys[i]);
                if (DT && !(power >= -7.994353375f)) continue;
                float alpha = ex2_approx_ftz(power);
                float weight = alpha * T[i][j];
                C[i][j][0] += rgb.x * weight;
                C[i][j][1] += rgb.y * weight;
                C[i][j][2] += rgb.z * weight;
                T[i][j] -= weight;
            }
    } else {
#pragma unroll
        for (int i = 0; i < TY; i++)
#pragma unroll
            for (int j = 0; j < TX; j++) {
                float dx = xy.x - (float)(ox + cb + j);
                float dy = xy.y - (float)(oy + rb + i);
                float power = co.w + co.x * dx * dx + co.z * dy * dy + co.y * dx * dy;
                float alpha = ex2_approx_ftz(power);
                C[i][j][0] += rgb.x * (alpha * T[i][j]);
                C[i][j][1] += rgb.y * (alpha * T[i][j]);
                C[i][j][2] += rgb.z * (alpha * T[i][j]);
                T[i][j] -= alpha * T[i][j];
            }
    }
}

// RANGE_MODE 0: ranges[] given; 1: warp search in the sorted keys.
// EXIT 0: the tile stops when all its pixels are saturated; EXIT 1: the top
// and bottom halves (8 rows each, lanes 0-15 and 16-31) stop independently,
// as the reference's two-warp split kernels do (renderCUDAWarpSplit,
// render.cu:4115-4357; renderCUDA32x16Split, render.cu:3859-4106).
// QUAD: the keys name 2x2 groups of 16x16 tiles (ranges and key ids count
// quads); each of a quad's four tiles is a work item of its own, whose warp
// blends, in list order, only the Gaussians whose value has that tile's bit,
// which is exactly the tile's per-tile list; the exit count runs over them.
template <int BX, int BY, int CADENCE, int SHADER, bool DT, int RANGE_MODE, bool TMA, bool BATCH, int EXIT = 0,
          bool QUAD = false>
__global__ __launch_bounds__(kRenderWarps * 32) void k_render(const RenderParams p)
{
    static_assert(!QUAD || (BX == 16 && BY == 16 && EXIT == 0 && !TMA), "quad renders: 16x16 tiles");
    constexpr int TX = BX / 8, TY = BY / 4;
    __shared__ WarpRing rings[kRenderWarps];
    const unsigned lane = threadIdx.x & 31u;
    const int warp = threadIdx.x >> 5;
    WarpRing& R = rings[warp];
    if (TMA) {
        if (lane == 0) {
            mbar_init(&R.bar[0], 1);
            mbar_init(&R.bar[1], 1);
            fence_mbar_init();
        }
        __syncwarp();
    }
    long long nl = p.d_num ? (long long)*p.d_num : (long long)p.n_host;
    const int n = (int)max(0LL, min(nl, p.cap));
    const int cb = (int)(lane & 7u) * TX;
    const int rb = (int)(lane >> 3) * TY;
    uint32_t phase_bits = 0;
    bool bad = false;
    bool timed_out = false;

    int item = blockIdx.x * kRenderWarps + warp;
    while (item < p.items) {
        const int tile = QUAD ? (item >> 2) : item;  // key tile id (a quad's id for QUAD)
        const int sub = item & 3;                     // QUAD: which tile of the quad
        // per-view geometry (batched renders); the single-view kernel reads
        // its parameters directly
        int W = 0, H = 0, gx = p.gx, ltile = tile;
        float3 bg = make_float3(0.f, 0.f, 0.f);
        uchar3* out = nullptr;
        if (BATCH) {
            // the view holding this global tile: last tile_base <= tile
            int lo = 0, hi = p.n_views - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (__ldg(&p.views[mid].tile_base) <= tile) lo = mid;
                else hi = mid - 1;
            }
            const RenderView& v = p.views[lo];
            W = v.W;
            H = v.H;
            gx = max(1, v.gx);
            ltile = tile - v.tile_base;
            bg = make_float3(v.bg[0], v.bg[1], v.bg[2]);
            out = reinterpret_cast<uchar3*>(v.out);
        }
        const int ox = QUAD ? (ltile % gx) * 32 + (sub & 1) * 16 : (ltile % gx) * BX;
        const int oy = QUAD ? (ltile / gx) * 32 + (sub >> 1) * 16 : (ltile / gx) * BY;
        if (QUAD && (ox >= (BATCH ? W : p.W) || oy >= (BATCH ? H : p.H))) {
            // a quad's tile beyond the image edge has no pixels and no Gaussians
            int next = 0;
            if (lane == 0) next = (int)atomicAdd(p.queue, 1u) + (int)gridDim.x * kRenderWarps;
            item = __shfl_sync(GSR_FULL_MASK, next, 0);
            continue;
        }
        const uint32_t sub_bit = QUAD ? (1u << (kQuadShift + sub)) : 0u;
        int start, end;
        if (RANGE_MODE == 0) {
            int2 r = make_int2(0, 0);
            if (lane == 0) r = __ldg(p.ranges + tile);
            // ranges come from the caller: keep them inside [0, n]
            start = min(max(__shfl_sync(GSR_FULL_MASK, r.x, 0), 0), n);
            end = min(max(__shfl_sync(GSR_FULL_MASK, r.y, 0), start), n);
        } else {
            start = warp_bound<false>(p.keys, 0, n, (uint32_t)tile, lane);
            end = warp_bound<true>(p.keys, start, n, (uint32_t)tile, lane);
        }
        float T[TY][TX];
        float C[TY][TX][3];
#pragma unroll
        for (int i = 0; i < TY; i++)
#pragma unroll
            for (int j = 0; j < TX; j++) {
                T[i][j] = 1.0f;
                C[i][j][0] = C[i][j][1] = C[i][j][2] = 0.0f;
            }
        const int total = end - start;
        bool blended_any = false;  // QUAD: the tile's own list is not empty
        if (total > 0) {
            int cur = 0;
            int scan = start;  // next list position to stage from
            int staged = stage_batch<TMA, QUAD>(R, 0, p, scan, end, lane, bad, sub_bit);
            int processed = 0;
            bool half_done = false;  // EXIT 1: this lane's half has stopped
            while (staged > 0) {
                const int bsize = staged;
                if (!wait_batch<TMA>(R, cur, phase_bits)) {
                    timed_out = true;
                    break;
                }
                const int nsize = scan < end ? stage_batch<TMA, QUAD>(R, cur ^ 1, p, scan, end, lane, bad, sub_bit)
                                             : 0;
                staged = nsize;
                blended_any = true;
                bool exit_now = false;
                for (int g = 0; g < bsize; g++) {
                    const float4 co = R.con[cur][g];
                    const float4 cd = R.rgbd[cur][g];
                    const float4 x2 = R.xy2[cur][g];
                    const float2 xy = R.sel[cur][g] ? make_float2(x2.z, x2.w) : make_float2(x2.x, x2.y);
                    if (EXIT == 0 || !half_done)
                        shade<TX, TY, SHADER, DT>(C, T, ox, oy, cb, rb, xy, co, make_float3(cd.x, cd.y, cd.z));
                    ++processed;
                    if (processed % CADENCE == 0) {
                        bool sat = true;
#pragma unroll
                        for (int i = 0; i < TY; i++)
#pragma unroll
                            for (int j = 0; j < TX; j++) sat = sat && T[i][j] < 0.0001f;
                        if (EXIT == 0) {
                            if (__all_sync(GSR_FULL_MASK, sat)) {
                                exit_now = true;
                                break;
                            }
                        } else {
                            const unsigned m = __ballot_sync(GSR_FULL_MASK, sat);
                            const bool lo = (m & 0xFFFFu) == 0xFFFFu, hi = (m >> 16) == 0xFFFFu;
                            if (lo && hi) {
                                exit_now = true;
                                break;
                            }
                            half_done = half_done || (lane < 16u ? lo : hi);
                        }
                    }
                }
                cur ^= 1;
                if (exit_now) {
                    // consume the batch already in flight so the ring is idle
                    if (nsize > 0 && !wait_batch<TMA>(R, cur, phase_bits)) timed_out = true;
                    break;
                }
            }
        }
        if (timed_out) break;
#pragma unroll
        for (int i = 0; i < TY; i++)
#pragma unroll
            for (int j = 0; j < TX; j++) {
                const int px = ox + cb + j, py = oy + rb + i;
                const bool any = QUAD ? blended_any : total > 0;
                if (BATCH) {
                    if (px < W && py < H) out[(size_t)py * W + px] = encode_px(C[i][j], T[i][j], any, bg);
                } else {
                    if (px < p.W && py < p.H) p.out[(size_t)py * p.W + px] = encode_px(C[i][j], T[i][j], any, p.bg);
                }
            }
        int next = 0;
        if (lane == 0) next = (int)atomicAdd(p.queue, 1u) + (int)gridDim.x * kRenderWarps;
        item = __shfl_sync(GSR_FULL_MASK, next, 0);
    }
    if (timed_out && lane == 0) record_error(p.status, kErrTimeout);
    if (__any_sync(GSR_FULL_MASK, bad) && lane == 0) record_error(p.status, kErrBadInput);
    if (TMA && timed_out) {
        // give copies still in flight a bounded chance to land before exit
        mbar_wait_bounded(&R.bar[0], (phase_bits >> 0) & 1u);
        mbar_wait_bounded(&R.bar[1], (phase_bits >> 1) & 1u);
    }
}

template <int BX, int BY, int CADENCE, int SHADER, bool DT, int RANGE_MODE, bool TMA, bool BATCH = false,
          int EXIT = 0, bool QUAD = false>
cudaError_t launch_variant(const RenderParams& p, cudaStream_t stream)
{
    auto kern = k_render<BX, BY, CADENCE, SHADER, DT, RANGE_MODE, TMA, BATCH, EXIT, QUAD>;
    // per device; host threads may race to fill it with the same value
    static std::atomic<int> per_sm_cache[kMaxDevices];
    const int dev = current_device();
    if (dev < 0) return cudaErrorInvalidDevice;
    int per_sm = per_sm_cache[dev].load(std::memory_order_relaxed);
    if (per_sm == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kRenderWarps * 32, 0) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        per_sm_cache[dev].store(per_sm, std::memory_order_relaxed);
    }
    const int warps_needed = p.items;
    int grid = device_sm_count() * per_sm;
    grid = max(1, min(grid, div_up(warps_needed, kRenderWarps)));
    kern<<<grid, kRenderWarps * 32, 0, stream>>>(p);
    return cudaGetLastError();
}

template <int BX, int BY>
cudaError_t dispatch_shape(int variant, bool tma, const RenderParams& p, cudaStream_t stream)
{
    constexpr int SH = (BX == 16 && BY == 16) ? 0 : 1;
    // FUSED/DEFAULT find their ranges in-kernel unless ranges were supplied
    // (the same [lower, upper) bounds, so the same image)
    const bool ranges = p.ranges != nullptr;
    switch (variant) {
    case GSR_RENDER_PERSISTENT_RANGES:
        return tma ? launch_variant<BX, BY, 8, 0, false, 0, true>(p, stream)
                   : launch_variant<BX, BY, 8, 0, false, 0, false>(p, stream);
    case GSR_RENDER_PERSISTENT_FUSED:
        if (ranges)
            return tma ? launch_variant<BX, BY, 16, 0, false, 0, true>(p, stream)
                       : launch_variant<BX, BY, 16, 0, false, 0, false>(p, stream);
        return tma ? launch_variant<BX, BY, 16, 0, false, 1, true>(p, stream)
                   : launch_variant<BX, BY, 16, 0, false, 1, false>(p, stream);
    case GSR_RENDER_DEFAULT:
        if (ranges)
            return tma ? launch_variant<BX, BY, 2, SH, false, 0, true>(p, stream)
                       : launch_variant<BX, BY, 2, SH, false, 0, false>(p, stream);
        return tma ? launch_variant<BX, BY, 2, SH, false, 1, true>(p, stream)
                   : launch_variant<BX, BY, 2, SH, false, 1, false>(p, stream);
    case GSR_RENDER_RANGES_CADENCE2:
        return tma ? launch_variant<BX, BY, 2, SH, false, 0, true>(p, stream)
                   : launch_variant<BX, BY, 2, SH, false, 0, false>(p, stream);
    case GSR_RENDER_DT:
        return tma ? launch_variant<BX, BY, 8, 0, true, 0, true>(p, stream)
                   : launch_variant<BX, BY, 8, 0, true, 0, false>(p, stream);
    case GSR_RENDER_SPLIT:  // axis-shared shader at every tile width, per-half exit
        if (BY != 16) return cudaErrorInvalidValue;
        if (ranges) return launch_variant<BX, BY, 2, 0, false, 0, false, false, 1>(p, stream);
        return launch_variant<BX, BY, 2, 0, false, 1, false, false, 1>(p, stream);
    default:
        return cudaErrorInvalidValue;
    }
}

// Quad renders (16x16 tiles, keys per 2x2 group of tiles; cp.async staging).
template <bool BATCH>
cudaError_t dispatch_quad(int variant, const RenderParams& p, cudaStream_t stream)
{
    const bool ranges = p.ranges != nullptr;
    switch (variant) {
    case GSR_RENDER_PERSISTENT_RANGES: return launch_variant<16, 16, 8, 0, false, 0, false, BATCH, 0, true>(p, stream);
    case GSR_RENDER_PERSISTENT_FUSED:
        if (ranges || BATCH) return launch_variant<16, 16, 16, 0, false, 0, false, BATCH, 0, true>(p, stream);
        return launch_variant<16, 16, 16, 0, false, 1, false, false, 0, true>(p, stream);
    case GSR_RENDER_DEFAULT:
        if (ranges || BATCH) return launch_variant<16, 16, 2, 0, false, 0, false, BATCH, 0, true>(p, stream);
        return launch_variant<16, 16, 2, 0, false, 1, false, false, 0, true>(p, stream);
    case GSR_RENDER_RANGES_CADENCE2: return launch_variant<16, 16, 2, 0, false, 0, false, BATCH, 0, true>(p, stream);
    case GSR_RENDER_DT: return launch_variant<16, 16, 8, 0, true, 0, false, BATCH, 0, true>(p, stream);
    default: return cudaErrorInvalidValue;
    }
}

// Batched renders: ranges always precomputed, cp.async staging, 16x16,
// 32x16 and 32x32 tiles.
template <int BX, int BY>
cudaError_t dispatch_batch(int variant, const RenderParams& p, cudaStream_t stream)
{
    constexpr int SH = (BX == 16 && BY == 16) ? 0 : 1;
    switch (variant) {
    case GSR_RENDER_PERSISTENT_RANGES: return launch_variant<BX, BY, 8, 0, false, 0, false, true>(p, stream);
    case GSR_RENDER_PERSISTENT_FUSED: return launch_variant<BX, BY, 16, 0, false, 0, false, true>(p, stream);
    case GSR_RENDER_DEFAULT:
    case GSR_RENDER_RANGES_CADENCE2: return launch_variant<BX, BY, 2, SH, false, 0, false, true>(p, stream);
    case GSR_RENDER_DT: return launch_variant<BX, BY, 8, 0, true, 0, false, true>(p, stream);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

static cudaError_t launch_prepared(const RenderArgs& a, RenderParams& p, cudaStream_t stream);

static bool use_render_tma()
{
    // per-thread cp.async staging measured faster than per-lane 16-byte bulk
    // copies (28 vs 48 us at 1080p, 2.5 vs 3.6 ms at 8K): bulk copies only on
    // request (read once, thread-safe initialisation)
    static const bool tma = [] {
        const char* e = getenv("GSR_RENDER_TMA");
        return e && strcmp(e, "1") == 0;
    }();
    return tma;
}

// ---------------------------------------------------------------------------
// Differentiable render (no counterpart in the reference): the forward of the
// persistent lite render (16x16 tiles, exit check every 8 Gaussians, same
// per-pixel arithmetic through shade<>) writing a float image, each pixel's
// final transmittance and each tile's number of blended Gaussians; and its
// backward, which walks every tile's list in reverse.

namespace {

constexpr int kTrainWarps = 4;
constexpr int kTrainCadence = 8;

struct TrainBatch {
    float2 xy[32];
    float4 con[32];
    float4 rgb[32];
    uint32_t gid[32];
    uint32_t use[32];  // the entry belongs to this tile (quad keys: its bit is set)
};

// Where tile (tx, ty) of `view` finds its list: its own range, or with quad
// keys its quad's range, whose entries carry the bit `qbit` when they
// belong to this tile.
__device__ __forceinline__ int train_list(const TrainRenderArgs& a, int view, int tile, int tx, int ty, int gx, int gy,
                                          uint32_t& qbit)
{
    qbit = 0u;
    if (!a.quad) return tile;
    const int qgx = quad_cols(gx), qpv = qgx * quad_cols(gy);
    qbit = 1u << (kQuadShift + ((tx & 1) | ((ty & 1) << 1)));
    return view * qpv + (ty >> 1) * qgx + (tx >> 1);
}

// One list entry: false when it is another tile's (quad keys), else its
// Gaussian in g.
__device__ __forceinline__ bool train_entry(const TrainRenderArgs& a, uint32_t v, uint32_t qbit, uint32_t& g)
{
    if (!a.quad) {
        g = v;
        return true;
    }
    g = v & kQuadGidMask;
    return (v & qbit) != 0u;
}

__global__ __launch_bounds__(kTrainWarps * 32) void k_render_train(const TrainRenderArgs a)
{
    __shared__ TrainBatch sb[kTrainWarps];
    const unsigned lane = threadIdx.x & 31u;
    const int warp = threadIdx.x >> 5;
    TrainBatch& B = sb[warp];
    // tile: global over the views; lt: within its view
    const int gx = (a.W + 15) / 16, gy = (a.H + 15) / 16, tiles = gx * gy;
    const int tile = blockIdx.x * kTrainWarps + warp;
    if (tile >= tiles * max(a.n_views, 1)) return;
    const int view = tile / tiles, lt = tile - view * tiles;
    const size_t pix0 = (size_t)view * a.W * a.H;
    const int n = (int)max(0LL, min((long long)*a.d_num, a.cap));
    const int tx = lt % gx, ty = lt / gx;
    const int ox = tx * 16, oy = ty * 16;
    const int cb = (int)(lane & 7u) * 2, rb = (int)(lane >> 3) * 4;
    uint32_t qbit;
    const int2 rg = __ldg(a.ranges + train_list(a, view, tile, tx, ty, gx, gy, qbit));
    const int start = min(max(rg.x, 0), n), end = min(max(rg.y, start), n);
    float T[4][2], C[4][2][3];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) {
            T[i][j] = 1.0f;
            C[i][j][0] = C[i][j][1] = C[i][j][2] = 0.0f;
        }
    // processed: Gaussians blended (the exit cadence counts these); used:
    // list positions up to the last one blended, what the backward replays
    int processed = 0, used = 0;
    bool exit_now = false;
    for (int pos = start; pos < end && !exit_now; pos += 32) {
        const int cnt = min(32, end - pos);
        __syncwarp();
        if ((int)lane < cnt) {
            uint32_t g;
            const bool mine = train_entry(a, __ldg(a.vals + pos + lane), qbit, g);
            B.use[lane] = mine ? 1u : 0u;
            if (mine && g < (uint32_t)a.P) {
                B.xy[lane] = __ldg(a.xy + g);
                B.con[lane] = __ldg(a.con + g);
                B.rgb[lane] = __ldg(a.rgbd + g);
            } else {  // another tile's, or outside the feature arrays: a transparent stand-in
                B.xy[lane] = make_float2(0.f, 0.f);
                B.con[lane] = make_float4(0.f, 0.f, 0.f, -1e30f);
                B.rgb[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
        __syncwarp();
        for (int k = 0; k < cnt; k++) {
            if (!B.use[k]) continue;
            const float4 rgb = B.rgb[k];
            shade<2, 4, 0, false>(C, T, ox, oy, cb, rb, B.xy[k], B.con[k], make_float3(rgb.x, rgb.y, rgb.z));
            ++processed;
            used = pos - start + k + 1;
            if (processed % kTrainCadence == 0) {
                bool sat = true;
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 2; j++) sat = sat && T[i][j] < 0.0001f;
                if (__all_sync(GSR_FULL_MASK, sat)) {
                    exit_now = true;
                    break;
                }
            }
        }
    }
    if (lane == 0) a.n_tile[tile] = used;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int px = ox + cb + j, py = oy + rb + i;
            if (px >= a.W || py >= a.H) continue;
            const size_t o = pix0 + (size_t)py * a.W + px;
            const float t = T[i][j], tt = t < 0.0001f ? 0.0f : t;
            a.T_final[o] = t;
            a.image[3 * o + 0] = C[i][j][0] + tt * a.bg[0];
            a.image[3 * o + 1] = C[i][j][1] + tt * a.bg[1];
            a.image[3 * o + 2] = C[i][j][2] + tt * a.bg[2];
        }
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(GSR_FULL_MASK, v, d);
    return v;
}

// Sums of eight values over the warp in 9 shuffles instead of 40: at each of
// the first three steps a lane keeps half of its partial sums and sends the
// other half to its partner.  Lane l returns the total of
// v[((l >> 4) & 1) * 4 + ((l >> 3) & 1) * 2 + ((l >> 2) & 1)], that is
// v[l >> 2] for every lane l with l & 3 == 0.
__device__ __forceinline__ float warp_sum8_spread(const float (&v)[8], unsigned lane)
{
    const bool b4 = (lane & 16u) != 0u, b3 = (lane & 8u) != 0u, b2 = (lane & 4u) != 0u;
    float h[4];
#pragma unroll
    for (int k = 0; k < 4; k++)
        h[k] = (b4 ? v[k + 4] : v[k]) + __shfl_xor_sync(GSR_FULL_MASK, b4 ? v[k] : v[k + 4], 16);
    float q[2];
#pragma unroll
    for (int k = 0; k < 2; k++)
        q[k] = (b3 ? h[k + 2] : h[k]) + __shfl_xor_sync(GSR_FULL_MASK, b3 ? h[k] : h[k + 2], 8);
    float t = (b2 ? q[1] : q[0]) + __shfl_xor_sync(GSR_FULL_MASK, b2 ? q[0] : q[1], 4);
    t += __shfl_xor_sync(GSR_FULL_MASK, t, 2);
    t += __shfl_xor_sync(GSR_FULL_MASK, t, 1);
    return t;
}

// Reverse traversal of each tile's blended Gaussians.  With T_after the
// transmittance behind Gaussian i and alpha_i recomputed bit for bit,
// T_before = T_after / (1 - alpha_i) (1 - alpha is exact once alpha >= 1/2);
// R, the colour composited behind i per unit transmittance, starts at bg (or
// 0 where the forward dropped the background term) and follows
// R <- alpha c + (1 - alpha) R.  Then
//   dL/dc_i     = sum_px alpha_i T_before dL/dC
//   dL/dalpha_i = T_before (c_i - R) . dL/dC,   d alpha/d power = alpha ln 2
// and the power's derivatives give the conic/opacity and centre gradients.
// The 9 per-Gaussian sums are reduced over the warp (eight of them spread
// over the lanes, warp_sum8_spread) and added atomically: by three lanes as
// 16-byte adds into the Gaussian's 12-float record (grad_rec), or by nine
// lanes into the three arrays.
// Five CTAs of 128 threads per SM (96 registers, a few bytes spilled): the
// kernel is bound by instruction issue with few warps resident, and the
// fifth CTA measured 1-2% faster per training step (8 views of 1 M Gaussians
// at 1280x720) than four at 120 registers.
__global__ __launch_bounds__(kTrainWarps * 32, 5) void k_render_backward(const TrainRenderArgs a)
{
    __shared__ TrainBatch sb[kTrainWarps];
    const unsigned lane = threadIdx.x & 31u;
    const int warp = threadIdx.x >> 5;
    TrainBatch& B = sb[warp];
    const int gx = (a.W + 15) / 16, gy = (a.H + 15) / 16, tiles = gx * gy;
    const int tile = blockIdx.x * kTrainWarps + warp;
    if (tile >= tiles * max(a.n_views, 1)) return;
    const int view = tile / tiles, lt = tile - view * tiles;
    const size_t pix0 = (size_t)view * a.W * a.H;
    const int n = (int)max(0LL, min((long long)*a.d_num, a.cap));
    const int tx = lt % gx, ty = lt / gx;
    const int ox = tx * 16, oy = ty * 16;
    const int cb = (int)(lane & 7u) * 2, rb = (int)(lane >> 3) * 4;
    uint32_t qbit;
    const int2 rg = __ldg(a.ranges + train_list(a, view, tile, tx, ty, gx, gy, qbit));
    const int start = min(max(rg.x, 0), n);
    const int count = min(max(__ldg(a.n_tile + tile), 0), max(0, min(max(rg.y, start), n) - start));
    float T[4][2], R[4][2][3], G[4][2][3];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int px = ox + cb + j, py = oy + rb + i;
            const bool in = px < a.W && py < a.H;
            const size_t o = in ? pix0 + (size_t)py * a.W + px : 0;
            const float t = in ? __ldg(a.T_final + o) : 1.0f;
            T[i][j] = t;
#pragma unroll
            for (int ch = 0; ch < 3; ch++) {
                R[i][j][ch] = t < 0.0001f ? 0.0f : a.bg[ch];
                G[i][j][ch] = in ? __ldg(a.grad_image + 3 * o + ch) : 0.0f;
            }
        }
    const float LN2 = 0.69314718055994531f;
    for (int hi = start + count; hi > start; hi -= 32) {
        const int lo = max(start, hi - 32), cnt = hi - lo;
        __syncwarp();
        if ((int)lane < cnt) {
            uint32_t g;
            const bool mine = train_entry(a, __ldg(a.vals + lo + lane), qbit, g);
            const bool ok = mine && g < (uint32_t)a.P;
            B.use[lane] = mine ? 1u : 0u;
            B.gid[lane] = ok ? g : 0xFFFFFFFFu;
            B.xy[lane] = ok ? __ldg(a.xy + g) : make_float2(0.f, 0.f);
            B.con[lane] = ok ? __ldg(a.con + g) : make_float4(0.f, 0.f, 0.f, -1e30f);
            B.rgb[lane] = ok ? __ldg(a.rgbd + g) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncwarp();
        for (int k = cnt - 1; k >= 0; k--) {
            if (!B.use[k]) continue;  // another tile of the quad
            const float2 xy = B.xy[k];
            const float4 co = B.con[k];
            const float4 c4 = B.rgb[k];
            const float col[3] = {c4.x, c4.y, c4.z};
            float gc[3] = {0.f, 0.f, 0.f};
            // dx depends on the column only and dy on the row only, so the
            // conic and centre gradients need three sums over this lane's
            // pixels of dp (per column, per row) and of dp * dx (per row)
            float s_col[2] = {0.f, 0.f}, g_w = 0.f, g_yy = 0.f, g_xy = 0.f, sy = 0.f, sx = 0.f;
            // the forward's per-pixel power, term for term (shade<>, SHADER 0)
            float xs[2], xc[2], dxs[2];
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const float dx = xy.x - (float)(ox + cb + j);
                dxs[j] = dx;
                xs[j] = co.x * dx * dx;
                xc[j] = co.y * dx;
            }
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float dy = xy.y - (float)(oy + rb + i);
                const float ys = co.z * dy * dy;
                float r = 0.f, q = 0.f;
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    const float power = fmaf(xc[j], dy, co.w + xs[j] + ys);
                    const float alpha = ex2_approx_ftz(power);
                    const float one_m = 1.0f - alpha;
                    const float Tb = one_m > 0.0f ? fminf(1.0f, T[i][j] / one_m) : T[i][j];
                    const float w = alpha * Tb;
                    float dalpha = 0.0f;
#pragma unroll
                    for (int ch = 0; ch < 3; ch++) {
                        const float d = col[ch] - R[i][j][ch];
                        gc[ch] = fmaf(w, G[i][j][ch], gc[ch]);
                        dalpha = fmaf(d, G[i][j][ch], dalpha);
                        R[i][j][ch] = fmaf(alpha, d, R[i][j][ch]);  // alpha c + (1 - alpha) R
                    }
                    T[i][j] = Tb;
                    // d power of this pixel, without its factor ln 2 (applied to the totals)
                    const float dp = dalpha * w;
                    r += dp;
                    q = fmaf(dp, dxs[j], q);
                    s_col[j] += dp;
                }
                g_w += r;
                g_yy = fmaf(dy * dy, r, g_yy);
                g_xy = fmaf(dy, q, g_xy);
                sy = fmaf(dy, r, sy);
                sx += q;
            }
            // d power / d (conic x, y, z, w) = (dx^2, dx dy, dy^2, 1);
            // d power / d centre = (2 co.x dx + co.y dy, 2 co.z dy + co.y dx)
            float v[8];
            v[0] = LN2 * fmaf(dxs[0] * dxs[0], s_col[0], dxs[1] * dxs[1] * s_col[1]);
            v[1] = LN2 * g_xy;
            v[2] = LN2 * g_yy;
            v[3] = LN2 * g_w;
            v[4] = LN2 * fmaf(2.0f * co.x, sx, co.y * sy);
            v[5] = LN2 * fmaf(2.0f * co.z, sy, co.y * sx);
            v[6] = gc[0];
            v[7] = gc[1];
            const float t8 = warp_sum8_spread(v, lane);
            const float t9 = warp_sum(gc[2]);
            // lanes 0, 4, .., 28 hold the totals of v[lane / 4]; every lane the ninth
            const uint32_t gid = B.gid[k];
            if (a.grad_rec) {
                // lane L < 3 adds slots 4L .. 4L + 3 of the Gaussian's record
                float r4[4];
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    const int slot = 4 * (int)(lane & 3u) + c;
                    const float x = __shfl_sync(GSR_FULL_MASK, t8, slot < 8 ? 4 * slot : 0);
                    r4[c] = slot < 8 ? x : (slot == 8 ? t9 : 0.0f);
                }
                if (lane < 3u && gid != 0xFFFFFFFFu)
                    atomicAdd(reinterpret_cast<float4*>(a.grad_rec + 12 * (size_t)gid) + lane,
                              make_float4(r4[0], r4[1], r4[2], r4[3]));
            } else if (gid != 0xFFFFFFFFu) {
                float* dst = nullptr;
                float val = t8;
                if ((lane & 3u) == 0u) {
                    const int q8 = (int)(lane >> 2);
                    dst = q8 < 4 ? a.grad_con + 4 * (size_t)gid + q8
                        : q8 < 6 ? a.grad_xy + 2 * (size_t)gid + (q8 - 4)
                                 : a.grad_rgb + 3 * (size_t)gid + (q8 - 6);
                } else if (lane == 1u) {
                    dst = a.grad_rgb + 3 * (size_t)gid + 2;
                    val = t9;
                }
                if (dst) atomicAdd(dst, val);
            }
        }
    }
}

}  // namespace

cudaError_t launch_render_train(const TrainRenderArgs& a, bool backward, cudaStream_t stream)
{
    const long long tiles = (long long)((a.W + 15) / 16) * ((a.H + 15) / 16) * max(a.n_views, 1);
    if (tiles <= 0) return cudaSuccess;
    if (tiles > INT32_MAX - kTrainWarps) return cudaErrorInvalidValue;
    const int grid = div_up((int)tiles, kTrainWarps);
    if (backward) k_render_backward<<<grid, kTrainWarps * 32, 0, stream>>>(a);
    else k_render_train<<<grid, kTrainWarps * 32, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_render(const RenderArgs& a, cudaStream_t stream)
{
    RenderParams p;
    p.n_host = a.num;
    p.d_num = a.d_num;
    p.cap = a.d_num ? a.cap : (long long)a.num;
    p.W = a.W;
    p.H = a.H;
    if (a.quad) {
        if (a.bx != 16 || a.by != 16) return cudaErrorInvalidValue;
        p.gx = quad_cols(div_up(a.W, 16));
        p.tiles = p.gx * quad_cols(div_up(a.H, 16));
        p.items = 4 * p.tiles;
    } else {
        p.gx = div_up(a.W, a.bx);
        p.tiles = p.gx * div_up(a.H, a.by);
        p.items = p.tiles;
    }
    p.P = a.P;
    p.xy = a.xy;
    p.rgbd = a.rgbd;
    p.con = a.con;
    p.keys = a.keys;
    p.vals = a.vals;
    p.ranges = a.ranges;
    p.bg = make_float3(a.bg[0], a.bg[1], a.bg[2]);
    p.out = reinterpret_cast<uchar3*>(a.out);
    p.queue = &a.ws->render_queue;
    p.status = &a.ws->status;
    p.views = nullptr;
    p.n_views = 0;
    return launch_prepared(a, p, stream);
}

cudaError_t launch_render_views(const RenderArgs& a, const RenderView* views_dev, int n_views, int total_tiles,
                                cudaStream_t stream)
{
    if (!views_dev || n_views <= 0) return cudaErrorInvalidValue;
    RenderParams p;
    p.n_host = a.num;
    p.d_num = a.d_num;
    p.cap = a.d_num ? a.cap : (long long)a.num;
    p.W = p.H = p.gx = 1;  // per view
    p.tiles = total_tiles;
    p.items = a.quad ? 4 * total_tiles : total_tiles;
    p.P = a.P;
    p.xy = a.xy;
    p.rgbd = a.rgbd;
    p.con = a.con;
    p.keys = a.keys;
    p.vals = a.vals;
    p.ranges = a.ranges;
    p.bg = make_float3(0.f, 0.f, 0.f);
    p.out = nullptr;
    p.queue = &a.ws->render_queue;
    p.status = &a.ws->status;
    p.views = views_dev;
    p.n_views = n_views;
    return launch_prepared(a, p, stream);
}

static cudaError_t launch_prepared(const RenderArgs& a, RenderParams& p, cudaStream_t stream)
{
    if (p.tiles <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(p.queue, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    // TMA bulk copies need 16-byte aligned feature arrays; GSR_RENDER_TMA=0
    // stages batches with per-thread cp.async copies instead.
    const bool tma = use_render_tma() && ((reinterpret_cast<uintptr_t>(a.xy) | reinterpret_cast<uintptr_t>(a.rgbd) |
                                           reinterpret_cast<uintptr_t>(a.con)) & 15u) == 0;
    if (p.views) {
        if (!p.ranges || ((reinterpret_cast<uintptr_t>(a.xy) | reinterpret_cast<uintptr_t>(a.rgbd) |
                           reinterpret_cast<uintptr_t>(a.con)) & 15u) != 0)
            return cudaErrorInvalidValue;
        if (a.quad) return a.bx == 16 && a.by == 16 ? dispatch_quad<true>(a.variant, p, stream) : cudaErrorInvalidValue;
        if (a.bx == 16 && a.by == 16) return dispatch_batch<16, 16>(a.variant, p, stream);
        if (a.bx == 32 && a.by == 16) return dispatch_batch<32, 16>(a.variant, p, stream);
        if (a.bx == 32 && a.by == 32) return dispatch_batch<32, 32>(a.variant, p, stream);
        return cudaErrorInvalidValue;
    }
    if (a.quad) return a.bx == 16 && a.by == 16 ? dispatch_quad<false>(a.variant, p, stream) : cudaErrorInvalidValue;
    if (a.bx == 16 && a.by == 16) return dispatch_shape<16, 16>(a.variant, tma, p, stream);
    if (a.bx == 32 && a.by == 16) return dispatch_shape<32, 16>(a.variant, tma, p, stream);
    if (a.bx == 24 && a.by == 16) return dispatch_shape<24, 16>(a.variant, tma, p, stream);
    if (a.bx == 32 && a.by == 32) return dispatch_shape<32, 32>(a.variant, tma, p, stream);
    return cudaErrorInvalidValue;
}

}  // namespace gsr
