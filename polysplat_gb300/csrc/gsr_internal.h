// Internal launch interfaces shared between the gsr translation units.
#pragma once

#include <cstddef>

#include "gsr_common.cuh"

namespace gsr {

// A Gaussian whose tile rectangle is large; its tiles are tested by a whole
// CTA in the second emission kernel.
struct MassiveEntry {
    float4 ctr_power_depth;  // centre x, centre y, power, depth (bits are the key's low word)
    float4 conic_gid;        // conic x, y, z, Gaussian index (bit pattern)
    int4 rect;               // tile rectangle [x0, x1) x [y0, y1)
};

// Two classes share one array: slots [0, huge_capacity) hold "huge"
// rectangles (swept by a whole CTA), the rest "large" ones (one warp each).
// A huge rectangle that finds its region full goes to the large region (a
// warp handles any size, only more slowly); one that finds both full is
// handled in place by its own warp in the preprocess.
struct MassiveQueue {
    MassiveEntry* entries;
    int capacity;        // total slots
    int huge_capacity;   // slots of the huge region
    uint32_t* count;     // [2] entries pushed: huge, large (may exceed the region: the rest went elsewhere)
    uint32_t* head;      // [2][2] entries taken: [pass][class]; pass 0 counts or emits keys, pass 1
                         // emits the depth-first pairs
    uint32_t* depth_hi;  // max depth bits of emitting Gaussians (for the sort's key compression)
};

// Tile id (and value) of a pair slot that a Gaussian's emission could not
// fill: the depth-first and ES emissions write exactly the counted number of
// pairs per Gaussian, padding with this id, which sorts after every real tile
// under any tile-id mask and which the tile ranges treat as past the end.
constexpr uint32_t kTileSentinel = 0xFFFFFFFFu;

// Per-Gaussian records of the depth-first pipeline's counting pass.
struct DepthFirstRecords {
    uint32_t* count;  // [P] number of tiles the Gaussian's keys go to
    uint32_t* dkey;   // [P] depth bit pattern (the key's low word)
    float4* geo;      // [P] conic x, y, z and power (the exact FP32 test inputs)
    int2* rect;       // [P] x0 | x1 << 16, y0 | y1 << 16; bit 31 of .y: queued as massive
    int ref_layout;   // nonzero: the reference's ES layout instead (rect = (x0 | y0 << 16, x1 | y1 << 16),
                      // depth FLT_MAX for culled Gaussians; no large-Gaussian queue)
};

struct PreprocessParams {
    MassiveQueue mq;
    DepthFirstRecords df;  // count mode only
    int P;
    const float* pos;
    const void* shs;
    const float* opacity;
    const float* cov3d;
    int W, H, bx, by, gx, gy;
    float view[16];  // column-major
    float proj[16];  // column-major
    float campos[3];
    float tanx, tany, fx, fy;
    float2* points_xy;
    float4* rgb_depth;
    float4* conic_opacity;
    uint64_t* keys;
    uint32_t* vals;
    long long cap;
    int* counter;
    // Batches of views (one launch over several views): a view's keys carry
    // tile ids offset by tile_base and values offset by gid_base; the
    // per-view parameter blocks live in device memory at `views`.
    int gid_base;
    int tile_base;
    const PreprocessParams* views;
    int n_views;  // entries at `views`
    // dispatch thresholds of the multi-tile emission (tiles of the rectangle)
    int massive_area;
    int huge_area;
    // Quad keys (bx = by = 16 only): one key per 2x2 group of tiles that the
    // Gaussian hits, with the quad's id as the key's tile id (quads numbered
    // row-major over ceil(gx / 2) columns) and the hit tiles as a 4-bit mask
    // in the value's top bits (see kQuadShift).
    int quad = 0;
    // Batches whose views all have the same P (views of one scene): block b
    // takes view b % n_views and block b / n_views of that view, so the
    // views' blocks over one range of Gaussians run side by side and the
    // range's parameters come from DRAM once and from L2 for the other views.
    int interleave = 0;
};
// Quad keys: bit (x & 1) | (y & 1) << 1 of value >> kQuadShift is set when
// the Gaussian hits tile (x, y) of the quad, by the same exact tile test the
// per-tile emission uses; the Gaussian's index is value & kQuadGidMask.
// So the Gaussians listed for one tile, in key order, are exactly that tile's
// per-tile list, while the sort handles one key per quad.
constexpr int kQuadShift = 28;
constexpr uint32_t kQuadGidMask = (1u << kQuadShift) - 1u;
__host__ __device__ inline int quad_cols(int gx) { return (gx + 1) >> 1; }

constexpr int kDefaultMassiveArea = 32;
constexpr int kDefaultHugeArea = 2048;

void camera_matrices(int W, int H, const float* pos, const float* rot, float fx, float fy, float zfar, float znear,
                     float* view, float* proj);
cudaError_t launch_preprocess(const PreprocessParams& p, bool half_sh, cudaStream_t stream);
// Parameter block of one single-view preprocess (what gsr_preprocess fills),
// with the large-Gaussian queue in the workspace when it is large enough.
gsr_status preprocess_params(PreprocessParams& p, int P, const float* pos, const void* shs, const float* opacity,
                             const float* cov3d, int width, int height, int block_x, int block_y,
                             const float* cam_pos, const float* cam_rot, float fx, float fy, float zfar, float znear,
                             float* points_xy, float* rgb_depth, float* conic_opacity, uint64_t* keys,
                             uint32_t* values, int64_t cap, int32_t* curr_offset, void* workspace,
                             size_t workspace_bytes);
// One preprocess (+ large-Gaussian emission) over n_views views whose
// parameter blocks are in device memory at base.views (shared fields --
// queue, keys, counter -- are the same in every block and in `base`).
// `blocks` covers the views' Gaussians one view after another (at least
// sum over views of ceil(P / 256)); blocks past the last view return at once.
cudaError_t launch_preprocess_views(const PreprocessParams& base, int n_views, int blocks, bool half_sh,
                                    cudaStream_t stream);
// Depth-first pipeline: counting pass (fills p.df, features and the massive
// queue), then the emission of a Gaussian's pairs at its offset (small
// rectangles and queued Gaussians separately).
cudaError_t launch_preprocess_count(const PreprocessParams& p, bool half_sh, cudaStream_t stream);
cudaError_t launch_df_emit_small(const PreprocessParams& p, const uint32_t* d_v, const uint32_t* sgids,
                                 const uint32_t* offsets, uint32_t* tiles, uint32_t* vals, long long cap,
                                 cudaStream_t stream);
cudaError_t launch_df_emit_massive(const PreprocessParams& p, const uint32_t* offsets, const uint32_t* rank,
                                   uint32_t* tiles, uint32_t* vals, long long cap, cudaStream_t stream);
cudaError_t launch_es_pass_b(int P, int bx, int by, int gx, const uint32_t* perm, const int32_t* cum,
                             const int32_t* count_sorted, const float2* xy, const float4* cpr, const int2* rb,
                             uint32_t* tiles, uint32_t* vals, long long cap, cudaStream_t stream);
cudaError_t launch_scene_prepare(int P, const float* log_scales, const float* quats, const float* logits,
                                 float* opacity, float* cov3d, cudaStream_t stream);

// ---- workspace layout ----------------------------------------------------
// [0, kHeaderBytes): header (status word, counters, histograms)
// then: sort alternate keys (8*cap), alternate values (4*cap), look-back
// state (passes * tiles * 256 * 4).
struct WorkspaceHeader {
    uint32_t status;          // OR of kErr* bits
    uint32_t render_queue;    // persistent render tile counter
    // preprocess region (cleared by every preprocess)
    uint32_t mq_count[2];     // massive-Gaussian queue: entries pushed per class
    uint32_t mq_head[2][2];   // massive-Gaussian queue: entries taken per pass and class
    uint32_t depth_hi;        // largest depth bit pattern of an emitting Gaussian
    uint32_t pad[7];
    // sort region (cleared by every sort)
    uint32_t pass_counter[8]; // per radix pass tile counter
    uint32_t hist[8][256];    // per-pass digit histograms
};
constexpr size_t kPreprocessRegionOffset = 2 * sizeof(uint32_t);
constexpr size_t kPreprocessRegionBytes = 7 * sizeof(uint32_t);
constexpr size_t kSortRegionOffset = 16 * sizeof(uint32_t);
constexpr size_t kHeaderBytes = 16384;
static_assert(sizeof(WorkspaceHeader) <= kHeaderBytes, "header too large");
static_assert(offsetof(WorkspaceHeader, mq_count) == kPreprocessRegionOffset &&
                  offsetof(WorkspaceHeader, pad) == kPreprocessRegionOffset + kPreprocessRegionBytes &&
                  offsetof(WorkspaceHeader, pass_counter) == kSortRegionOffset,
              "header layout");

// Massive-Gaussian queue capacity of a workspace (entries of 48 bytes); the
// queue sits right after the header.  Gaussians beyond it are emitted in
// place by their own warp (slower, same keys).
constexpr int kMassiveQueueEntries = 1 << 20;  // 48 MB: a 4K view of a 10 M-Gaussian scene queues ~10^6
constexpr int kMassiveHugeEntries = 1 << 15;
constexpr size_t kMassiveQueueBytes = (size_t)kMassiveQueueEntries * sizeof(MassiveEntry);
// Small workspace for preprocess-only and render-only calls.
constexpr size_t kSmallWorkspaceBytes = kHeaderBytes + kMassiveQueueBytes;

constexpr int kSortThreads = 512;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096 keys per tile
constexpr int kMaxPasses = 8;

size_t sort_workspace_bytes(long long cap);
// Tile-range area at the end of a full workspace (frames of up to
// kWorkspaceRangeTiles tiles; the fused forward uses it when the caller
// passes no ranges buffer).
constexpr int kWorkspaceRangeTiles = 1 << 20;
int2* workspace_ranges(void* ws, long long cap);

// Lower bound of the depth bit patterns of emitted keys: view depth is > 0.2
// (preprocess.cu:363), so every key's low word exceeds the bits of 0.2f.
constexpr uint32_t kDepthBitsFloor = 0x3E4CCCCDu;

struct SortArgs {
    int num;                // host count (used when d_num == nullptr)
    const int32_t* d_num;   // device count or nullptr
    long long cap;          // capacity of the key buffers
    int end_bit;
    // Depth compression (fused forward only): order by
    // (tile << nb) | (low word - kDepthBitsFloor) with nb = bits(depth_hi -
    // floor), taken from the workspace header the preprocess filled.  Same
    // order as the full key for every key the preprocess emits.
    bool compress_depth;
    const uint64_t* keys_in;
    const uint32_t* vals_in;
    uint64_t* keys_out;
    uint32_t* vals_out;
    void* ws;
    size_t ws_bytes;
};
cudaError_t launch_sort(const SortArgs& a, cudaStream_t stream);

// Generic sort plumbing (also used by the depth-first pipeline).
enum : int {
    kOrderMasked = 0,             // key & mask(end_bit)
    kOrderDepthCompressed64 = 1,  // (tile << nb) | (low word - floor), nb from the header's depth_hi
    kOrderDepth32 = 2,            // 32-bit depth bits - floor, width from the header's depth_hi
};
struct OrderMap {
    int kind;
    int end_bit;
    // digits at or above this bit of the order word hold tile ids; where a key
    // holds both depth and tile digits those passes rank with per-bit
    // ballots, which beat match.any on them (kOrderDepthCompressed64 takes the
    // boundary from the depth width on the device)
    int tile_from_bit = 64;
};
struct SortScratch {
    WorkspaceHeader* hdr;  // counters, histograms, status, depth_hi
    void* alt_keys;
    uint32_t* alt_vals;
    uint32_t* look[2];
    long long tiles_cap;
};
size_t sort_scratch_bytes(long long cap, int key_bytes);
SortScratch carve_sort_scratch(WorkspaceHeader* hdr, void* mem, long long cap, int key_bytes);
SortScratch workspace_sort_scratch(void* ws, long long cap);
cudaError_t launch_sort32(int num, const int32_t* d_num, long long cap, OrderMap order, int max_passes,
                          const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                          const SortScratch& s, cudaStream_t stream);
cudaError_t launch_sort64(int num, const int32_t* d_num, long long cap, OrderMap order, int max_passes,
                          const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out, uint32_t* vals_out,
                          const SortScratch& s, cudaStream_t stream);

cudaError_t launch_tile_ranges(int num, const int32_t* d_num, long long cap, int tiles, const uint64_t* keys,
                               int32_t* ranges, bool scan_semantics, cudaStream_t stream);
// Same, over sorted 32-bit tile ids.
cudaError_t launch_tile_ranges32(const int32_t* d_num, long long cap, int tiles, const uint32_t* tile_ids,
                                 int2* ranges, cudaStream_t stream);
cudaError_t launch_gather(int num, const int32_t* d_num, const uint32_t* values, const float2* sxy,
                          const float4* srgbd, const float4* scon, float2* dxy, float4* drgbd, float4* dcon,
                          long long cap, cudaStream_t stream);

struct RenderArgs {
    int variant;
    int num;
    const int32_t* d_num;
    long long cap;  // key-buffer capacity: the device count is clamped to it
    int W, H, bx, by;
    int P;
    const float2* xy;
    const float4* rgbd;
    const float4* con;
    const uint64_t* keys;
    const uint32_t* vals;
    const int2* ranges;
    float bg[3];
    uint8_t* out;
    WorkspaceHeader* ws;
    int quad = 0;  // keys and ranges per 2x2 group of 16x16 tiles (PreprocessParams::quad)
};
cudaError_t launch_render(const RenderArgs& a, cudaStream_t stream);

// Differentiable render (16x16 tiles, lite exit cadence 8): the forward
// writes `image` (float [H,W,3]), `T_final` ([H,W]) and `n_tile` ([tiles]);
// the backward reads them with `grad_image` and accumulates the per-Gaussian
// gradients of xy [P,2], conic/opacity [P,4] and colour [P,3].  With
// n_views > 1 the views (all W x H) follow one another: tile t of view v is
// global tile v * tiles + t in `ranges` and `n_tile`, and the per-pixel
// buffers are [n_views, H, W(, 3)]; P then counts the feature rows of all
// views.
struct TrainRenderArgs {
    int W, H, P;
    int n_views;  // 0 or 1: one view
    // quad keys: ranges are per 2x2 group of tiles (view * quads + quad) and
    // values carry the hit tiles in their top bits; n_tile then counts list
    // positions up to the last Gaussian blended, not Gaussians
    int quad;
    const int32_t* d_num;
    long long cap;
    const uint32_t* vals;
    const int2* ranges;
    const float2* xy;
    const float4* rgbd;
    const float4* con;
    float bg[3];
    float* image;
    float* T_final;
    int32_t* n_tile;
    const float* grad_image;
    float* grad_xy;
    float* grad_con;
    float* grad_rgb;
    // when set, replaces the three arrays above: one 12-float record per
    // feature row, conic/opacity (4), xy (2), colour (3) and 3 unused, added
    // to with three 16-byte atomics
    float* grad_rec;
};
cudaError_t launch_render_train(const TrainRenderArgs& a, bool backward, cudaStream_t stream);

// One view of a batched render: its tiles are [tile_base, tile_base +
// gx * gy) of the batch's global tile ids (quads, with gx quads per row, for
// quad renders).
struct RenderView {
    int tile_base;
    int gx;
    int W, H;
    float bg[3];
    int pad;
    uint8_t* out;  // [H, W, 3]
};
// Render every tile of n_views views (view blocks in device memory, sorted
// by tile_base, views_dev[0].tile_base == 0) in one persistent launch.
// a.W/a.H are ignored; total_tiles = sum of the views' tile counts.
cudaError_t launch_render_views(const RenderArgs& a, const RenderView* views_dev, int n_views, int total_tiles,
                                cudaStream_t stream);

// Depth-first forward (depthfirst.cu): scratch of P-sized arrays, and the
// pipeline from the counting pass to the tile ranges.  The emitted pair count
// goes to p.counter; tile ids and values land in tile_keys_out / vals_out.
size_t df_scratch_bytes(int P);
cudaError_t launch_depth_first(const PreprocessParams& p, bool half_sh, void* scratch, size_t scratch_bytes,
                               WorkspaceHeader* hdr, const SortScratch& tile_sort, int tiles, uint32_t* tile_keys_in,
                               uint32_t* vals_in, uint32_t* tile_keys_out, uint32_t* vals_out, int2* ranges,
                               cudaStream_t stream);

int device_sm_count();
// Per-device host caches (occupancy, attribute set-up) hold kMaxDevices
// entries; current_device() is the current device, or -1 when the query
// fails or the index is beyond the caches.
constexpr int kMaxDevices = 64;
int current_device();

// Failure-detection hooks (gsr_debug_*): the look-back spin bound the next
// sorts use (kSpinLimit unless a test lowered it), and whether the first
// digit pass of the next sorts leaves tile 0 untaken, so that every later
// tile's look-back waits on an entry nobody publishes.
uint32_t sort_wait_limit();
bool sort_stall_first_tile();

// Stage-timing hook (gsr_set_profile_events): records the next caller-owned
// event on `stream` when profiling is on; no-op otherwise.
void profile_mark(cudaStream_t stream);

}  // namespace gsr
