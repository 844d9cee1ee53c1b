// Batched forward: several views -- of different scenes and resolutions --
// rendered by one pass of the pipeline.  No counterpart in the reference
// (it renders one view per call).
//
// Every view contributes its Gaussians to one preprocess launch (one grid
// row per view), its keys to one key buffer (tile ids offset by the view's
// first global tile, values by the view's first feature slot), one radix sort
// over all keys, one tile-range pass and one persistent render launch over
// the tiles of all views.  Small views therefore share launches instead of
// each leaving most of the GPU idle.
//
// The per-view parameter blocks live in device memory: they are packed on
// the host into a pinned staging slot and copied to the device ahead of the
// kernels.  The kernel sequence depends only on the batch's shape (views,
// preprocess blocks over all views, total tiles, tile shape, variant), so it is
// captured once per shape into a CUDA graph and replayed for any cameras,
// scenes of the same size class and output buffers.
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "gsr_internal.h"

namespace gsr {
namespace {

constexpr int kStagingSlots = 4;

struct Shape {
    int variant, half, bx, by, n_views, blocks, tiles, quad;  // tiles: key tile ids (quads when quad)
    bool operator<(const Shape& o) const
    {
        return std::tie(variant, half, bx, by, n_views, blocks, tiles, quad) <
               std::tie(o.variant, o.half, o.bx, o.by, o.n_views, o.blocks, o.tiles, o.quad);
    }
};

// Preprocess blocks of a batch, rounded up so that batches of similar size
// share a captured graph (the extra blocks return at once).
constexpr int kBlockBucket = 512;

}  // namespace
}  // namespace gsr

struct gsr_batcher {
    int device = 0;
    int max_views = 0;
    long long cap = 0;
    long long max_gaussians = 0;
    int max_tiles = 0;
    // device buffers (owned)
    void* ws = nullptr;
    size_t ws_bytes = 0;
    uint64_t *ku = nullptr, *ks = nullptr;
    uint32_t *vu = nullptr, *vs = nullptr;
    float2* xy = nullptr;
    float4 *rgbd = nullptr, *con = nullptr;
    int2* ranges = nullptr;
    int32_t* counter = nullptr;
    gsr::PreprocessParams* d_pre = nullptr;
    gsr::RenderView* d_views = nullptr;
    // pinned staging: parameter blocks of a batch, one slot per batch in flight
    unsigned char* h_stage = nullptr;
    size_t slot_bytes = 0;
    cudaEvent_t slot_done[gsr::kStagingSlots] = {};
    int next_slot = 0;
    // captured kernel sequences per batch shape
    std::map<gsr::Shape, cudaGraphExec_t> graphs;
    std::map<gsr::Shape, int> seen;
    std::mutex mu;
    int last_total = 0;
    int massive_area = gsr::kDefaultMassiveArea;
    int huge_area = gsr::kDefaultHugeArea;
};

namespace gsr {
namespace {

size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

struct Sizes {
    size_t ws, keys, vals, xy, f4, ranges, pre, views, total;
};

Sizes sizes_of(int max_views, long long cap, long long max_g, int max_tiles)
{
    Sizes s;
    s.ws = al(sort_workspace_bytes(cap));
    s.keys = al((size_t)cap * 8);
    s.vals = al((size_t)cap * 4);
    s.xy = al((size_t)max_g * 8);
    s.f4 = al((size_t)max_g * 16);
    s.ranges = al((size_t)max_tiles * 8);
    s.pre = al((size_t)max_views * sizeof(PreprocessParams));
    s.views = al((size_t)max_views * sizeof(RenderView));
    s.total = s.ws + 2 * s.keys + 2 * s.vals + s.xy + 2 * s.f4 + s.ranges + s.pre + s.views + 256;
    return s;
}

bool valid_shape(int bx, int by) { return (bx == 16 && by == 16) || (bx == 32 && by == 16) || (bx == 32 && by == 32); }

// Fill the parameter block of one view (the same fields the single-view
// preprocess entry fills), plus its offsets into the batch.
void pack_view(PreprocessParams& p, const gsr_scene_ref& sc, const gsr_view& v, int bx, int by, bool quad,
               gsr_batcher* b, int gid_base, int tile_base)
{
    std::memset(&p, 0, sizeof(p));
    WorkspaceHeader* h = reinterpret_cast<WorkspaceHeader*>(b->ws);
    p.mq.entries = reinterpret_cast<MassiveEntry*>(reinterpret_cast<char*>(b->ws) + kHeaderBytes);
    p.mq.capacity = kMassiveQueueEntries;
    p.mq.huge_capacity = kMassiveHugeEntries;
    p.mq.count = h->mq_count;
    p.mq.head = &h->mq_head[0][0];
    p.mq.depth_hi = &h->depth_hi;
    p.P = sc.P;
    p.pos = sc.pos;
    p.shs = sc.shs;
    p.opacity = sc.opacity;
    p.cov3d = sc.cov3d;
    p.W = v.width;
    p.H = v.height;
    p.bx = bx;
    p.by = by;
    p.gx = div_up(v.width, bx);
    p.gy = div_up(v.height, by);
    camera_matrices(v.width, v.height, v.cam_pos, v.cam_rot, v.focal_x, v.focal_y, v.z_far, v.z_near, p.view,
                    p.proj);
    p.campos[0] = v.cam_pos[0];
    p.campos[1] = v.cam_pos[1];
    p.campos[2] = v.cam_pos[2];
    p.tanx = v.width / (2.0f * v.focal_x);
    p.tany = v.height / (2.0f * v.focal_y);
    p.fx = v.focal_x;
    p.fy = v.focal_y;
    // features of view i start at its first feature slot
    p.points_xy = b->xy + gid_base;
    p.rgb_depth = b->rgbd + gid_base;
    p.conic_opacity = b->con + gid_base;
    p.keys = b->ku;
    p.vals = b->vu;
    p.cap = b->cap;
    p.counter = b->counter;
    p.gid_base = gid_base;
    p.tile_base = tile_base;
    p.views = b->d_pre;
    p.n_views = 0;  // set per batch in the base block
    p.massive_area = b->massive_area;
    p.huge_area = b->huge_area;
    p.quad = quad ? 1 : 0;
}

// The kernel sequence of a batch (everything after the parameter copy).
cudaError_t enqueue(gsr_batcher* b, const Shape& s, cudaStream_t st)
{
    WorkspaceHeader* h = reinterpret_cast<WorkspaceHeader*>(b->ws);
    cudaError_t e = cudaMemsetAsync(&h->status, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->counter, 0, sizeof(int32_t), st);
    if (e != cudaSuccess) return e;
    PreprocessParams base;
    std::memset(&base, 0, sizeof(base));
    base.mq.entries = reinterpret_cast<MassiveEntry*>(reinterpret_cast<char*>(b->ws) + kHeaderBytes);
    base.mq.capacity = kMassiveQueueEntries;
    base.mq.huge_capacity = kMassiveHugeEntries;
    base.mq.count = h->mq_count;
    base.mq.head = &h->mq_head[0][0];
    base.mq.depth_hi = &h->depth_hi;
    base.keys = b->ku;
    base.vals = b->vu;
    base.cap = b->cap;
    base.counter = b->counter;
    base.views = b->d_pre;
    base.n_views = s.n_views;
    base.bx = s.bx;
    base.by = s.by;
    base.quad = s.quad;
    e = launch_preprocess_views(base, s.n_views, s.blocks, s.half != 0, st);
    if (e != cudaSuccess) return e;
    SortArgs sa;
    sa.num = 0;
    sa.d_num = b->counter;
    sa.cap = b->cap;
    sa.end_bit = 32 + bits_for((uint32_t)s.tiles);
    sa.compress_depth = true;
    sa.keys_in = b->ku;
    sa.vals_in = b->vu;
    sa.keys_out = b->ks;
    sa.vals_out = b->vs;
    sa.ws = b->ws;
    sa.ws_bytes = b->ws_bytes;
    if ((e = launch_sort(sa, st)) != cudaSuccess) return e;
    e = launch_tile_ranges(0, b->counter, b->cap, s.tiles, b->ks, reinterpret_cast<int32_t*>(b->ranges), false, st);
    if (e != cudaSuccess) return e;
    RenderArgs ra;
    std::memset(&ra, 0, sizeof(ra));
    ra.variant = s.variant;
    ra.num = 0;
    ra.d_num = b->counter;
    ra.cap = b->cap;
    ra.W = ra.H = 1;
    ra.bx = s.bx;
    ra.by = s.by;
    ra.P = (int)b->max_gaussians;
    ra.xy = b->xy;
    ra.rgbd = b->rgbd;
    ra.con = b->con;
    ra.keys = b->ks;
    ra.vals = b->vs;
    ra.ranges = b->ranges;
    ra.ws = h;
    ra.quad = s.quad;
    return launch_render_views(ra, b->d_views, s.n_views, s.tiles, st);
}

}  // namespace
}  // namespace gsr

using namespace gsr;

extern "C" {

size_t gsr_batcher_device_bytes(int max_views, int64_t key_capacity, int64_t max_gaussians, int max_tiles)
{
    if (max_views <= 0 || key_capacity <= 0 || max_gaussians <= 0 || max_tiles <= 0) return 0;
    return sizes_of(max_views, key_capacity, max_gaussians, max_tiles).total;
}

gsr_batcher* gsr_batcher_create(int max_views, int64_t key_capacity, int64_t max_gaussians, int max_tiles)
{
    if (max_views <= 0 || max_views > 32767 || key_capacity <= 0 || key_capacity >= (1LL << 30) ||
        max_gaussians <= 0 || max_gaussians >= (1LL << 31) || max_tiles <= 0 || max_tiles > (1 << 26))
        return nullptr;
    gsr_batcher* b = new gsr_batcher();
    cudaGetDevice(&b->device);
    b->max_views = max_views;
    b->cap = key_capacity;
    b->max_gaussians = max_gaussians;
    b->max_tiles = max_tiles;
    const Sizes s = sizes_of(max_views, key_capacity, max_gaussians, max_tiles);
    char* base = nullptr;
    if (cudaMalloc(&base, s.total) != cudaSuccess) {
        delete b;
        return nullptr;
    }
    size_t o = 0;
    auto take = [&](size_t n) {
        char* q = base + o;
        o += n;
        return q;
    };
    b->ws = take(s.ws);
    b->ws_bytes = s.ws;
    b->ku = reinterpret_cast<uint64_t*>(take(s.keys));
    b->ks = reinterpret_cast<uint64_t*>(take(s.keys));
    b->vu = reinterpret_cast<uint32_t*>(take(s.vals));
    b->vs = reinterpret_cast<uint32_t*>(take(s.vals));
    b->xy = reinterpret_cast<float2*>(take(s.xy));
    b->rgbd = reinterpret_cast<float4*>(take(s.f4));
    b->con = reinterpret_cast<float4*>(take(s.f4));
    b->ranges = reinterpret_cast<int2*>(take(s.ranges));
    b->d_pre = reinterpret_cast<PreprocessParams*>(take(s.pre));
    b->d_views = reinterpret_cast<RenderView*>(take(s.views));
    b->counter = reinterpret_cast<int32_t*>(take(256));
    b->slot_bytes = al(s.pre) + al(s.views);
    // The zero fill runs on the legacy default stream, which streams created
    // non-blocking (every torch stream) do not wait for: it must be finished
    // before any stream uses the block.  A batch launched on such a stream
    // while the fill still ran had its parameter blocks cleared under it, and
    // its kernels read null scene and image pointers.
    bool ok = cudaMemset(base, 0, s.total) == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess &&
              cudaMallocHost(&b->h_stage, b->slot_bytes * kStagingSlots) == cudaSuccess;
    for (int i = 0; ok && i < kStagingSlots; i++)
        ok = cudaEventCreateWithFlags(&b->slot_done[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        gsr_batcher_destroy(b);
        return nullptr;
    }
    return b;
}

void gsr_batcher_destroy(gsr_batcher* b)
{
    if (!b) return;
    cudaDeviceSynchronize();
    for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
    for (int i = 0; i < kStagingSlots; i++)
        if (b->slot_done[i]) cudaEventDestroy(b->slot_done[i]);
    if (b->h_stage) cudaFreeHost(b->h_stage);
    if (b->ws) cudaFree(b->ws);  // the first carve: base of the whole block
    delete b;
}

gsr_status gsr_batcher_render(gsr_batcher* b, int variant, int shs_half, int block_x, int block_y,
                              const gsr_scene_ref* scenes, int n_scenes, const gsr_view* views, int n_views,
                              int use_graph, gsr_stream_t stream)
{
    if (!b || !scenes || !views || n_views <= 0 || n_views > b->max_views || n_scenes <= 0) return GSR_INVALID_ARG;
    const bool quad = (variant & GSR_QUAD_KEYS) != 0;  // one key per 2x2 group of 16x16 tiles
    variant &= ~GSR_QUAD_KEYS;
    if (!valid_shape(block_x, block_y) || variant < 0 || variant > GSR_RENDER_DT) return GSR_INVALID_ARG;
    if (quad && (block_x != 16 || block_y != 16 || b->max_gaussians > (long long)kQuadGidMask + 1))
        return GSR_INVALID_ARG;
    // key tile ids of one view: its tiles, or its quads
    auto key_tiles = [&](int w, int h, int& gx) {
        gx = quad ? quad_cols(div_up(w, 16)) : div_up(w, block_x);
        return gx * (quad ? quad_cols(div_up(h, 16)) : div_up(h, block_y));
    };
    cudaStream_t st = (cudaStream_t)stream;
    std::lock_guard<std::mutex> lk(b->mu);
    // layout of the batch: first feature slot and first tile of every view
    long long g = 0;
    int tiles = 0, blocks = 0;
    for (int i = 0; i < n_views; i++) {
        const gsr_view& v = views[i];
        if (v.scene < 0 || v.scene >= n_scenes || v.width <= 0 || v.height <= 0 || !v.out) return GSR_INVALID_ARG;
        const gsr_scene_ref& sc = scenes[v.scene];
        if (sc.P < 0 || (sc.P > 0 && (!sc.pos || !sc.shs || !sc.opacity || !sc.cov3d))) return GSR_INVALID_ARG;
        if (div_up(v.width, block_x) >= 65536) return GSR_INVALID_ARG;
        g += sc.P;
        int gxv = 0;
        tiles += key_tiles(v.width, v.height, gxv);
        blocks += div_up(sc.P, 256);
        if (g > b->max_gaussians || tiles > b->max_tiles) return GSR_INVALID_ARG;
    }
    // pack the parameter blocks into a free staging slot
    const int slot = b->next_slot;
    b->next_slot = (slot + 1) % kStagingSlots;
    if (cudaEventSynchronize(b->slot_done[slot]) != cudaSuccess) return GSR_CUDA_ERROR;
    unsigned char* stage = b->h_stage + (size_t)slot * b->slot_bytes;
    PreprocessParams* hp = reinterpret_cast<PreprocessParams*>(stage);
    RenderView* hv = reinterpret_cast<RenderView*>(stage + al((size_t)b->max_views * sizeof(PreprocessParams)));
    long long gb = 0;
    int tb = 0;
    for (int i = 0; i < n_views; i++) {
        const gsr_view& v = views[i];
        const gsr_scene_ref& sc = scenes[v.scene];
        pack_view(hp[i], sc, v, block_x, block_y, quad, b, (int)gb, tb);
        RenderView& rv = hv[i];
        rv.tile_base = tb;
        const int vt = key_tiles(v.width, v.height, rv.gx);
        rv.W = v.width;
        rv.H = v.height;
        rv.bg[0] = v.bg[0];
        rv.bg[1] = v.bg[1];
        rv.bg[2] = v.bg[2];
        rv.pad = 0;
        rv.out = v.out;
        gb += sc.P;
        tb += vt;
    }
    cudaError_t e = cudaMemcpyAsync(b->d_pre, hp, (size_t)n_views * sizeof(PreprocessParams), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_views, hv, (size_t)n_views * sizeof(RenderView), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaEventRecord(b->slot_done[slot], st);
    if (e != cudaSuccess) return GSR_CUDA_ERROR;
    b->last_total = tiles;

    const Shape s{variant, shs_half ? 1 : 0, block_x, block_y, n_views,
                  div_up(blocks > 0 ? blocks : 1, kBlockBucket) * kBlockBucket, tiles, quad ? 1 : 0};
    if (!use_graph || st == nullptr) {
        e = enqueue(b, s, st);
        return e == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
    }
    auto it = b->graphs.find(s);
    if (it == b->graphs.end()) {
        // the first batch of a shape runs eagerly (one-time kernel attribute
        // and occupancy queries happen outside any capture); the second is
        // captured and every later one replays the graph
        if (b->seen[s]++ == 0) {
            e = enqueue(b, s, st);
            return e == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
        }
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return GSR_CUDA_ERROR;
        const cudaError_t ce = enqueue(b, s, st);
        const cudaError_t ee = cudaStreamEndCapture(st, &graph);
        if (ce != cudaSuccess || ee != cudaSuccess || !graph) {
            if (graph) cudaGraphDestroy(graph);
            return GSR_CUDA_ERROR;
        }
        cudaGraphExec_t exec = nullptr;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return GSR_CUDA_ERROR;
        it = b->graphs.emplace(s, exec).first;
    }
    e = cudaGraphLaunch(it->second, st);
    return e == cudaSuccess ? GSR_OK : GSR_CUDA_ERROR;
}

gsr_status gsr_batcher_finish(gsr_batcher* b, int32_t* num_rendered, gsr_stream_t stream)
{
    if (!b) return GSR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t status = 0;
    int32_t n = 0;
    if (cudaStreamSynchronize(st) != cudaSuccess) return GSR_CUDA_ERROR;
    if (cudaMemcpy(&status, b->ws, sizeof(status), cudaMemcpyDeviceToHost) != cudaSuccess) return GSR_CUDA_ERROR;
    if (cudaMemcpy(&n, b->counter, sizeof(n), cudaMemcpyDeviceToHost) != cudaSuccess) return GSR_CUDA_ERROR;
    if (num_rendered) *num_rendered = n;
    if (status & kErrTimeout) return GSR_TIMEOUT;
    if (n > b->cap || (status & kErrOverflow)) return GSR_OVERFLOW;
    return GSR_OK;
}

int gsr_batcher_graphs(const gsr_batcher* b) { return b ? (int)b->graphs.size() : 0; }

gsr_status gsr_batcher_set_thresholds(gsr_batcher* b, int massive_area, int huge_area)
{
    if (!b || massive_area < 2 || huge_area < massive_area) return GSR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(b->mu);
    b->massive_area = massive_area;
    b->huge_area = huge_area;
    return GSR_OK;
}

const int32_t* gsr_batcher_counter(const gsr_batcher* b) { return b ? b->counter : nullptr; }

const uint32_t* gsr_batcher_status(const gsr_batcher* b)
{
    return b ? reinterpret_cast<const uint32_t*>(b->ws) : nullptr;
}

}  // extern "C"
