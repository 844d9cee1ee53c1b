/*
 * gsr -- GB300-native 3D Gaussian Splatting forward rasterizer: C ABI.
 *
 * Plain pointers, sizes and a cudaStream_t; no framework types.  Every entry
 * point is asynchronous on the given stream and returns GSR_OK,
 * GSR_INVALID_ARG or GSR_CUDA_ERROR for launch-time problems.  Errors found on
 * the device (key-buffer overflow, a bounded wait that expired) are recorded
 * in the status word of the caller's workspace and are turned into a
 * gsr_status by gsr_read_status().
 *
 * Each entry point replaces one launcher of the reference rasterizer
 * (LuoLongZan/PolySplat, csrc/ops.h); the citation is given beside it.
 * Device arrays use the reference layouts:
 *   pos [P,3] f32, shs [P,48] f32 or f16 (interleaved [P,16,3]),
 *   opacity [P] f32, cov3d [P,6] f32 (xx,xy,xz,yy,yz,zz),
 *   points_xy [P,2] f32, rgb_depth [P,4] f32, conic_opacity [P,4] f32,
 *   keys u64 = tile << 32 | float_bits(view depth), values u32 = Gaussian index,
 *   ranges int32 [tiles,2], image uint8 [H,W,3].
 * Camera position (3 floats) and rotation (3x3 row-major camera-to-world, as
 * in cameras.json) and the background colour are HOST pointers, read on the
 * host exactly as the reference's bindings do (csrc/pybind.cpp:131-143).
 */
#ifndef GSR_H_
#define GSR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* gsr_stream_t; /* == cudaStream_t */

typedef enum {
    GSR_OK = 0,
    GSR_OVERFLOW = 1,      /* more keys than the key buffer holds; true count reported */
    GSR_TIMEOUT = 2,       /* a bounded device-side wait expired */
    GSR_INVALID_ARG = 3,
    GSR_CUDA_ERROR = 4,
} gsr_status;

/* Render variants: the blend of every variant name the reference exposes
 * maps onto one of these (tile size, exit-check cadence, range source). */
typedef enum {
    GSR_RENDER_PERSISTENT_RANGES = 0, /* render_16x16_preranges_smem_persistent_lite (render.cu:1717-1864): cadence 8 */
    GSR_RENDER_PERSISTENT_FUSED = 1,  /* ..._lite_fused (render.cu:2026-2174): ranges found in-kernel, cadence 16 */
    GSR_RENDER_DEFAULT = 2,           /* render_16x16 / renderCUDA (render.cu:2176): ranges in-kernel, cadence 2 */
    GSR_RENDER_RANGES_CADENCE2 = 3,   /* preranges variants with per-pair exit checks */
    GSR_RENDER_DT = 4,                /* ..._lite_dt (render.cu:1871-2018): skips power < log2(1/255), cadence 8 */
    GSR_RENDER_SPLIT = 5,             /* render_{16,24,32}x16_split (render.cu:3859-4357): ranges in-kernel, cadence 2,
                                         top and bottom 8-row halves stop independently; 16-row tiles only */
} gsr_render_variant;

/* Flag OR-ed into the variant of gsr_forward, gsr_forward_depth_first and
 * gsr_batcher_render (16x16 tiles; not with GSR_RENDER_SPLIT).  No counterpart in the reference: the
 * sort handles one key per 2x2 group of 16x16 tiles ("quad") instead of one
 * per tile.  A key's tile id names the quad (quads numbered row-major,
 * ceil(ceil(W/16)/2) per row); bits 28-31 of its value mark which of the
 * quad's tiles, (x & 1) | (y & 1) << 1, the Gaussian hits by the per-tile
 * emission's own test, and bits 0-27 hold the Gaussian's index (so P must be
 * below 2^28).  The render blends each 16x16 tile from the Gaussians with
 * its bit, in key order, which is that tile's per-tile list: the image is
 * the per-tile pipeline's, with fewer keys to sort.  The key and value
 * buffers then hold quad keys, not the reference's per-tile keys. */
#define GSR_QUAD_KEYS 0x100

/* Library version and a check that a CUDA device of compute capability 10.3
 * is present (returns GSR_CUDA_ERROR otherwise). */
int gsr_version(void);
gsr_status gsr_device_check(int device);

/* ---- workspace ---------------------------------------------------------- */
/* Bytes of device workspace for a frame whose key buffer holds `capacity`
 * keys: radix-sort ping-pong buffers and look-back state, the tile-queue
 * counter and the status word.  Replaces get_sort_buffer_size
 * (csrc/cuda_rasterizer/sort.cu:127-149, csrc/pybind.cpp:346-349); the
 * workspace is the reference's `list_sorting_space`. */
size_t gsr_workspace_size(int64_t capacity);
/* Small workspace (status word, render tile queue, large-Gaussian queue) for
 * preprocess-only and render-only calls. */
size_t gsr_render_workspace_size(void);
/* Clear the workspace's status word (asynchronous). */
gsr_status gsr_workspace_reset(void* workspace, gsr_stream_t stream);
/* Synchronise `stream`, read the status word and the key counter, and map
 * them to a status.  *num_out receives the true key count (it may exceed
 * capacity, in which case GSR_OVERFLOW is returned). */
gsr_status gsr_read_status(const void* workspace, const int32_t* d_num, int64_t capacity, int32_t* num_out,
                           gsr_stream_t stream);

/* View and projection matrices (column-major float[16]) the preprocess uses
 * for a camera; host-side, no GPU work.  Replaces getViewMatrix /
 * getProjectionMatrix (csrc/cuda_rasterizer/preprocess.cu:643-671). */
void gsr_camera_matrices(int width, int height, const float* cam_pos, const float* cam_rot, float focal_x,
                         float focal_y, float z_far, float z_near, float* view16, float* proj16);

/* ---- scene preparation -------------------------------------------------- */
/* Raw INRIA parameters -> render inputs: opacity = sigmoid(logit),
 * cov3d = R S^2 R^T (upper triangle) with S = exp(log_scales) and R from the
 * normalised w-first quaternion.  Replaces the CPU loop of loadPly_torch /
 * computeCov3D (csrc/pybind.cpp:22-56, 105-117). */
gsr_status gsr_scene_prepare(int P, const float* log_scales, const float* quats, const float* opacity_logits,
                             float* opacity, float* cov3d, gsr_stream_t stream);

/* ---- preprocess ---------------------------------------------------------- */
/* Projection, EWA conic, degree-3 SH colour, culling and tile-key emission.
 * Keys are appended at *curr_offset (atomically); writes past
 * key_capacity are dropped but counted.  shs_half != 0 selects FP16 SH.
 * `workspace` (at least gsr_render_workspace_size() bytes, or NULL) holds
 * the queue of Gaussians with large tile rectangles, which a second kernel
 * spreads over whole CTAs; without it those are emitted by their own warp
 * (same keys, slower).  Replaces preprocess / preprocess_half_sh
 * (csrc/ops.h:42-48, 104-111; csrc/cuda_rasterizer/preprocess.cu:1252-1330;
 * csrc/pybind.cpp:122-181). */
gsr_status gsr_preprocess(int P, const float* pos, const void* shs, int shs_half, const float* opacity,
                          const float* cov3d, int width, int height, int block_x, int block_y,
                          const float* cam_pos, const float* cam_rot, float focal_x, float focal_y, float z_far,
                          float z_near, float* points_xy, float* rgb_depth, float* conic_opacity, uint64_t* keys,
                          uint32_t* values, int64_t key_capacity, int32_t* curr_offset, void* workspace,
                          size_t workspace_bytes, gsr_stream_t stream);

/* ---- sort ----------------------------------------------------------------- */
/* Stable ascending LSD radix sort of (u64 key, u32 value) pairs over bits
 * [0, 32 + bits(tiles)).  The count is *d_num when d_num != NULL (device
 * resident, no host sync), else num.  keys_in/values_in are preserved.
 * Replaces sort_gaussian (csrc/cuda_rasterizer/sort.cu:107-125,
 * csrc/pybind.cpp:333-344). */
gsr_status gsr_sort(int num, const int32_t* d_num, int width, int height, int block_x, int block_y,
                    void* workspace, size_t workspace_bytes, const uint64_t* keys_in, const uint32_t* values_in,
                    uint64_t* keys_out, uint32_t* values_out, int64_t capacity, gsr_stream_t stream);

/* Same sort over an explicit bit range [0, end_bit), end_bit in 1..64. */
gsr_status gsr_sort_bits(int num, const int32_t* d_num, int end_bit, void* workspace, size_t workspace_bytes,
                         const uint64_t* keys_in, const uint32_t* values_in, uint64_t* keys_out,
                         uint32_t* values_out, int64_t capacity, gsr_stream_t stream);

/* Same sort as gsr_sort_bits, with no workspace argument and no allocation:
 * no counterpart in the reference.  For callers that cannot allocate or
 * hold device scratch (a thin FFI host that owns only the key/value buffers;
 * latency-bound loops that must not call cudaMalloc, which can synchronise
 * the device).  Scratch is a library-owned static device array sized for
 * capacity <= 262144 pairs; larger capacities return GSR_INVALID_ARG.  The
 * first call on each device looks up that array's address (make it before
 * any stream capture on that device) and keeps it for the life of the
 * process, so it is not for use after cudaDeviceReset on that device.  All
 * calls share the array: calls that overlap in time race and must be
 * serialised by the caller. */
gsr_status gsr_sort_bits_static(int num, const int32_t* d_num, int end_bit, const uint64_t* keys_in,
                                const uint32_t* values_in, uint64_t* keys_out, uint32_t* values_out,
                                int64_t capacity, gsr_stream_t stream);
/* Device-side outcome of the last gsr_sort_bits_static on `stream`: waits for
 * the stream and reads the static array's status word (no allocation).
 * GSR_TIMEOUT when a bounded look-back wait ran out (the output is then not
 * sorted), else GSR_OK.  The word is shared like the array: read it before
 * the next static sort starts.  No counterpart in the reference. */
gsr_status gsr_sort_bits_static_status(gsr_stream_t stream);

/* ---- tile ranges / gather ----------------------------------------------- */
/* ranges[t] = [first, end) of tile t in the sorted keys.  scan_semantics = 0
 * reproduces precompute_tile_ranges (binary search: empty tiles get
 * start == end == lower bound; render.cu:10-35, 3510-3521, 6812-6824);
 * scan_semantics = 1 reproduces precompute_tile_ranges_scan (empty tiles get
 * {0,0}; render.cu:3526-3557, 6826-6845). */
gsr_status gsr_tile_ranges(int num, const int32_t* d_num, int width, int height, int block_x, int block_y,
                           const uint64_t* keys_sorted, int32_t* ranges, int scan_semantics, gsr_stream_t stream);

/* dst[i] = src[values[i]] for xy, rgb_depth and conic_opacity.  Replaces
 * gather_features (csrc/cuda_rasterizer/gather.cu:46-58, pybind.cpp:351-364). */
gsr_status gsr_gather(int num, const int32_t* d_num, const uint32_t* values, const float* src_xy,
                      const float* src_rgb_depth, const float* src_conic, float* dst_xy, float* dst_rgb_depth,
                      float* dst_conic, gsr_stream_t stream);

/* ---- render ------------------------------------------------------------- */
/* Persistent tile-queue blend: one warp per tile, 32-Gaussian batches staged
 * into shared memory by TMA bulk copies under mbarrier double-buffering,
 * whole-tile early exit by warp vote, truncating uint8 encode.
 * `ranges` is required for the *_RANGES/DT variants, `keys_sorted` for the
 * FUSED/DEFAULT variants.  P is the length of the feature arrays (bounds).
 * block_x/block_y select the tile shape (16x16, 24x16, 32x16, 32x32).
 * Replaces render_16x16* / render_32x16* / render_32x32 / render_24x16_split
 * (csrc/cuda_rasterizer/render.cu:4365-4385, 6445-6652; csrc/ops.h:164-354). */
gsr_status gsr_render(int variant, int num, const int32_t* d_num, int width, int height, int block_x, int block_y,
                      int P, const float* points_xy, const float* rgb_depth, const float* conic_opacity,
                      const uint64_t* keys_sorted, const uint32_t* values_sorted, const int32_t* ranges,
                      const float* bg_color, uint8_t* out_color, void* workspace, gsr_stream_t stream);

/* ---- fused forward ------------------------------------------------------ */
/* preprocess -> sort -> [ranges] -> render in one call, with the key count
 * kept on the device (no host synchronisation; capturable in a CUDA graph).
 * `ranges` may be NULL for the FUSED/DEFAULT variants.  Replaces
 * forward_fused / forward_fused_e2e / forward_fused_e2e_preranges /
 * sort_and_render (csrc/pybind.cpp:876-1149). */
gsr_status gsr_forward(int variant, int P, const float* pos, const void* shs, int shs_half, const float* opacity,
                       const float* cov3d, int width, int height, int block_x, int block_y, const float* cam_pos,
                       const float* cam_rot, float focal_x, float focal_y, float z_far, float z_near,
                       int32_t* curr_offset, void* workspace, size_t workspace_bytes, uint64_t* keys_unsorted,
                       uint32_t* values_unsorted, uint64_t* keys_sorted, uint32_t* values_sorted,
                       int64_t key_capacity, float* points_xy, float* rgb_depth, float* conic_opacity,
                       int32_t* ranges, const float* bg_color, uint8_t* out_color, gsr_stream_t stream);

/* ---- depth-first forward ------------------------------------------------ */
/* The reference's "early sorting" two-pass pipeline
 * (csrc/cuda_rasterizer/preprocess.cu:673-1248, sort.cu:151-285,
 * example.py:246-291) as one call: a counting pass, a depth sort of the
 * Gaussians that hit a tile, emission of (tile, Gaussian) pairs in depth
 * order, a stable sort of the 32-bit tile ids, tile ranges and the render.
 * Same image as gsr_forward; pairs with equal tile and equal depth bits keep
 * Gaussian index order.  `scene_scratch` holds gsr_depth_first_scratch_size(P)
 * bytes of per-Gaussian arrays.  On return tiles_sorted / values_sorted hold
 * the sorted pairs, `ranges` (or, when NULL, the workspace's range area) the
 * tile ranges, and *curr_offset the pair count M (M > key_capacity:
 * overflow, reported by gsr_read_status).  Any variant; ranges are always
 * precomputed. */
size_t gsr_depth_first_scratch_size(int P);
gsr_status gsr_forward_depth_first(int variant, int P, const float* pos, const void* shs, int shs_half,
                                   const float* opacity, const float* cov3d, int width, int height, int block_x,
                                   int block_y, const float* cam_pos, const float* cam_rot, float focal_x,
                                   float focal_y, float z_far, float z_near, int32_t* curr_offset, void* workspace,
                                   size_t workspace_bytes, void* scene_scratch, size_t scene_scratch_bytes,
                                   uint32_t* tiles_unsorted, uint32_t* values_unsorted, uint32_t* tiles_sorted,
                                   uint32_t* values_sorted, int64_t key_capacity, float* points_xy, float* rgb_depth,
                                   float* conic_opacity, int32_t* ranges, const float* bg_color, uint8_t* out_color,
                                   gsr_stream_t stream);

/* ---- ES ("early sorting") steps ------------------------------------------- */
/* The reference's ES helper operators one by one, with its buffer layouts
 * (csrc/pybind.cpp:183-330).  Pointers are device pointers except cam_pos
 * and cam_rot (host).
 *
 * gsr_es_pass_a replaces preprocess_es_pass_a{,_half_sh}
 * (csrc/cuda_rasterizer/preprocess.cu:673-992): the preprocess's features,
 * plus per Gaussian tiles_per_gauss [P] (hit tiles, 0 when culled),
 * conic_power_raw [P,4] (conic a, b, c and power), depth_natural [P] (view z,
 * FLT_MAX when culled) and rect_bounds [P,2] (rect_min, rect_max packed as
 * x | y << 16).
 *
 * gsr_es_depth_sort_and_scan replaces es_depth_sort_and_scan (sort.cu:185-245):
 * identity = 0..P-1, (depth_sorted, perm) = stable sort of (depth_natural,
 * identity), tiles_per_gauss_sorted = tiles_per_gauss[perm], cum_offsets_sorted
 * = its exclusive scan, *total_out (device) = the pair count.  sort_space is
 * a workspace of at least gsr_workspace_size(P) bytes, scan_space
 * gsr_es_scan_buffer_size(P) bytes.
 *
 * gsr_es_pass_b replaces preprocess_es_pass_b (preprocess.cu:993-1248): for
 * the s-th Gaussian in depth order, its pairs (tile id y * grid_x + x,
 * Gaussian index) in tile row-major order from cum_offsets_sorted[s] on.
 * Pairs at or past `capacity` are not written.
 *
 * gsr_es_tile_sort replaces es_tile_sort (sort.cu:247-285): stable sort of the
 * num pairs by tile id over the bit width of the tile count, and
 * keys_sorted_out[i] = tile_keys_sorted[i] << 32 for the range search.
 * sort_space holds at least gsr_workspace_size(num) bytes. */
gsr_status gsr_es_pass_a(int P, const float* pos, const void* shs, int shs_half, const float* opacity,
                         const float* cov3d, int width, int height, int block_x, int block_y, const float* cam_pos,
                         const float* cam_rot, float focal_x, float focal_y, float z_far, float z_near,
                         float* points_xy, float* rgb_depth, float* conic_opacity, int32_t* tiles_per_gauss,
                         float* conic_power_raw, float* depth_natural, int32_t* rect_bounds, gsr_stream_t stream);
size_t gsr_es_scan_buffer_size(int P);
gsr_status gsr_es_depth_sort_and_scan(int P, const int32_t* tiles_per_gauss, const float* depth_natural,
                                      uint32_t* identity, uint32_t* perm, float* depth_sorted,
                                      int32_t* tiles_per_gauss_sorted, int32_t* cum_offsets_sorted,
                                      int32_t* total_out, void* sort_space, size_t sort_bytes, void* scan_space,
                                      size_t scan_bytes, gsr_stream_t stream);
gsr_status gsr_es_pass_b(int P, int width, int height, int block_x, int block_y, const uint32_t* perm,
                         const int32_t* cum_offsets_sorted, const int32_t* tiles_per_gauss_sorted,
                         const float* points_xy, const float* conic_power_raw, const int32_t* rect_bounds,
                         uint32_t* tile_keys_unsorted, uint32_t* values_unsorted, int64_t capacity,
                         gsr_stream_t stream);
gsr_status gsr_es_tile_sort(int num, int width, int height, int block_x, int block_y, const uint32_t* tile_keys_unsorted,
                            const uint32_t* values_unsorted, uint32_t* tile_keys_sorted, uint32_t* values_sorted,
                            uint64_t* keys_sorted_out, void* sort_space, size_t sort_bytes, gsr_stream_t stream);

/* ---- tile order (reordered-render helpers) --------------------------------- */
/* gsr_tile_order replaces compute_tile_order, compute_tile_order_packed and
 * compute_tile_order_packed_morton (render.cu:6959-7087; pybind.cpp:461-553):
 * tile_ids[t] = t; tile_order = the tiles by descending sort key, equal keys
 * in index order; tile_counts = the sorted keys.  The key is the tile's pair
 * count (ranges[t].y - ranges[t].x), or with morton_bucket > 0
 * (min(count / morton_bucket, 0xFFFF) << 16) | (0xFFFF - Morton(x, y) & 0xFFFF)
 * (render.cu:4496-4520).  With tile_desc != NULL, tile_desc[i] = {col, row,
 * start, end} of tile_order[i]; with zigzag_group > 1 the odd groups of
 * zigzag_group positions take their slice of the order backwards
 * (render.cu:4813-4866).  temp holds gsr_tile_order_temp_size(total_tiles)
 * bytes (= get_tile_order_sort_temp_size). */
size_t gsr_tile_order_temp_size(int total_tiles);
gsr_status gsr_tile_order(const int32_t* tile_ranges, int total_tiles, int x_blocks, int morton_bucket,
                          int zigzag_group, int32_t* tile_desc, uint32_t* tile_order, uint32_t* tile_counts,
                          uint32_t* tile_ids, void* temp, size_t temp_bytes, gsr_stream_t stream);
/* Per-tile ranges back from descriptors: ranges[row * x_blocks + col] =
 * {start, end} (what the reordered renders read; the tile order never
 * changes a tile's pixels). */
gsr_status gsr_tile_desc_ranges(const int32_t* tile_desc, int total_tiles, int x_blocks, int32_t* tile_ranges,
                                gsr_stream_t stream);

/* ---- batched forward ------------------------------------------------------ */
/* No counterpart in the reference, which renders one view per call.  Views
 * of different scenes and resolutions are rendered by one pass of the
 * pipeline: one preprocess launch over all views, one radix sort over all
 * keys (tile ids offset per view), one tile-range pass and one persistent
 * render launch over every view's tiles.  The per-view parameters are copied
 * to the device ahead of the kernels, so the kernel sequence of a batch
 * shape (number of views, largest scene in 256-Gaussian blocks, total tiles,
 * tile shape, variant) is captured once into a CUDA graph (use_graph != 0,
 * non-default stream) and replayed for new cameras and outputs. */
typedef struct {
    int P;
    const float* pos;      /* [P,3] */
    const void* shs;       /* [P,48] f32 or f16 (shs_half) */
    const float* opacity;  /* [P] */
    const float* cov3d;    /* [P,6] */
} gsr_scene_ref;

typedef struct {
    int scene;             /* index into the scene array */
    int width, height;
    float cam_pos[3];      /* host values, as gsr_forward's cam_pos / cam_rot */
    float cam_rot[9];
    float focal_x, focal_y, z_far, z_near;
    float bg[3];
    uint8_t* out;          /* device [height, width, 3] */
} gsr_view;

typedef struct gsr_batcher gsr_batcher;

/* Device bytes a batcher allocates at creation (keys, workspace, features,
 * ranges, parameter blocks); nothing is allocated per batch. */
size_t gsr_batcher_device_bytes(int max_views, int64_t key_capacity, int64_t max_gaussians, int max_tiles);
/* NULL on bad sizes or allocation failure.  max_gaussians bounds the sum of
 * the views' scene sizes in one batch, max_tiles the sum of their tiles. */
gsr_batcher* gsr_batcher_create(int max_views, int64_t key_capacity, int64_t max_gaussians, int max_tiles);
void gsr_batcher_destroy(gsr_batcher* b);
/* Enqueue one batch on `stream` (tile shape 16x16, 32x16 or 32x32).  Asynchronous;
 * the images are complete when the stream reaches this point. */
gsr_status gsr_batcher_render(gsr_batcher* b, int variant, int shs_half, int block_x, int block_y,
                              const gsr_scene_ref* scenes, int n_scenes, const gsr_view* views, int n_views,
                              int use_graph, gsr_stream_t stream);
/* Synchronise `stream` and report the last batch: GSR_OVERFLOW when its keys
 * exceeded key_capacity (*num_rendered = true count). */
gsr_status gsr_batcher_finish(gsr_batcher* b, int32_t* num_rendered, gsr_stream_t stream);
/* Graphs captured so far; device addresses of the batch's key counter and
 * status word (for asynchronous read-back). */
int gsr_batcher_graphs(const gsr_batcher* b);
const int32_t* gsr_batcher_counter(const gsr_batcher* b);
const uint32_t* gsr_batcher_status(const gsr_batcher* b);
/* Dispatch thresholds of the tile-key emission, in tiles of a Gaussian's
 * rectangle: from massive_area (default 32) on, a rectangle is queued for the
 * large-Gaussian kernel; from huge_area (default 2048) on, a whole CTA sweeps
 * it.  They change which scheme tests the tiles, never the keys. */
gsr_status gsr_batcher_set_thresholds(gsr_batcher* b, int massive_area, int huge_area);

/* ---- differentiable render -------------------------------------------------- */
/* No counterpart in the reference, which renders only.  The forward takes raw
 * parameters (means [P,3], log-scales [P,3], w-first quaternions [P,4],
 * opacity logits [P], SH [P,48] f32), runs the scene transform, preprocess,
 * sort and tile ranges at 16x16 tiles, and renders a float image [H,W,3]
 * together with what the backward replays: each pixel's final transmittance
 * T_final [H,W] and each tile's number of blended Gaussians n_tile [tiles].
 * The sorted values, ranges, features and those two buffers must be kept for
 * the backward, which takes dL/dimage and writes (accumulate = 0) or adds
 * (accumulate != 0) the gradients of every raw parameter; grad_xy [P,2],
 * grad_con [P,4] and grad_rgb [P,3] are its scratch.  Read the key count and
 * status with gsr_read_status after the forward (GSR_OVERFLOW: grow
 * key_capacity and run it again). */
gsr_status gsr_train_forward(int P, const float* means, const float* log_scales, const float* quats,
                             const float* logits, const float* shs, int width, int height, const float* cam_pos,
                             const float* cam_rot, float focal_x, float focal_y, float z_far, float z_near,
                             const float* bg_color, float* opacity, float* cov3d, int32_t* curr_offset,
                             void* workspace, size_t workspace_bytes, uint64_t* keys_unsorted,
                             uint32_t* values_unsorted, uint64_t* keys_sorted, uint32_t* values_sorted,
                             int64_t key_capacity, float* points_xy, float* rgb_depth, float* conic_opacity,
                             int32_t* ranges, int32_t* n_tile, float* T_final, float* image, gsr_stream_t stream);
gsr_status gsr_train_backward(int P, const float* means, const float* log_scales, const float* quats,
                              const float* logits, const float* shs, int width, int height, const float* cam_pos,
                              const float* cam_rot, float focal_x, float focal_y, float z_far, float z_near,
                              const float* bg_color, const int32_t* curr_offset, int64_t key_capacity,
                              const uint32_t* values_sorted, const int32_t* ranges, const int32_t* n_tile,
                              const float* T_final, const float* points_xy, const float* rgb_depth,
                              const float* conic_opacity, const float* grad_image, float* grad_xy, float* grad_con,
                              float* grad_rgb, float* g_means, float* g_log_scales, float* g_quats, float* g_logits,
                              float* g_shs, int accumulate, gsr_stream_t stream);
/* The same over n_views cameras of one scene, all width x height, in one
 * pass: one preprocess launch over every view, one sort over all keys (tile
 * ids view * tiles + tile, values view * P + Gaussian), one tile-range pass,
 * one render and one render backward over every view's tiles, and one
 * preprocess adjoint per 16 views that sums the views' gradients per
 * Gaussian.  Cameras are host arrays: cam_pos [n_views,3], cam_rot
 * [n_views,9] and cam_intr [n_views,4] = (focal_x, focal_y, z_far, z_near).
 * Per-view buffers follow one another: features [n_views*P, ...], ranges
 * and n_tile [n_views*tiles], T_final [n_views,H,W], image and grad_image
 * [n_views,H,W,3].  The backward's scratch grad_feat [n_views*P, 12]
 * (16-byte aligned) holds one record per feature row: the gradients of
 * conic/opacity (4), xy (2) and colour (3), and 3 unused.  view_scratch is
 * device memory of gsr_train_views_scratch_bytes(n_views) for the views'
 * parameter blocks; it must stay untouched until the forward has run.
 * flags = GSR_QUAD_KEYS (both calls alike) sorts one key per 2x2 group of
 * tiles (n_views * P below 2^28): ranges then hold one entry per quad
 * (view * quads + quad), n_tile counts each tile's list positions up to its
 * last blended Gaussian, and the images are those of per-tile keys. */
size_t gsr_train_views_scratch_bytes(int n_views);
gsr_status gsr_train_forward_views(int P, const float* means, const float* log_scales, const float* quats,
                                   const float* logits, const float* shs, int n_views, int width, int height,
                                   const float* cam_pos, const float* cam_rot, const float* cam_intr,
                                   const float* bg_color, float* opacity, float* cov3d, void* view_scratch,
                                   size_t view_scratch_bytes, int32_t* curr_offset, void* workspace,
                                   size_t workspace_bytes, uint64_t* keys_unsorted, uint32_t* values_unsorted,
                                   uint64_t* keys_sorted, uint32_t* values_sorted, int64_t key_capacity,
                                   float* points_xy, float* rgb_depth, float* conic_opacity, int32_t* ranges,
                                   int32_t* n_tile, float* T_final, float* image, int flags, gsr_stream_t stream);
gsr_status gsr_train_backward_views(int P, const float* means, const float* log_scales, const float* quats,
                                    const float* logits, const float* shs, int n_views, int width, int height,
                                    const float* cam_pos, const float* cam_rot, const float* cam_intr,
                                    const float* bg_color, const int32_t* curr_offset, int64_t key_capacity,
                                    const uint32_t* values_sorted, const int32_t* ranges, const int32_t* n_tile,
                                    const float* T_final, const float* points_xy, const float* rgb_depth,
                                    const float* conic_opacity, const float* grad_image, float* grad_feat,
                                    float* g_means, float* g_log_scales, float* g_quats, float* g_logits,
                                    float* g_shs, int accumulate, int flags, gsr_stream_t stream);

/* ---- stage timing ------------------------------------------------------- */
/* Profiling hook with no counterpart in the reference.  After
 * gsr_profile_begin(frames), each of the next `frames` gsr_forward calls
 * records library-owned CUDA events on its stream before the preprocess and
 * after every stage (preprocess, sort upsweep, each radix pass, tile ranges
 * when the variant needs them, render).  gsr_profile_read() synchronises and
 * writes the stage durations in ms, row f = frame f, `max_stages` columns,
 * and returns the number of stages per frame (or -1).  gsr_profile_end()
 * stops recording and frees the events.  The recording state is
 * process-wide: one session at a time, driven from one host thread. */
gsr_status gsr_profile_begin(int frames);
int gsr_profile_read(float* ms, int frames, int max_stages);
void gsr_profile_end(void);

/* Text of the last CUDA error seen by the library (for diagnostics). */
const char* gsr_last_error(void);

/* ---- failure-detection hooks ---------------------------------------------- */
/* No counterpart in the reference.  Process-wide switches that let a test
 * make a bounded device wait run out, so that the timeout path can be checked
 * on a GPU without faulting or hanging it.  gsr_debug_set_sort_wait_limit
 * sets how many times the radix sort's look-back re-reads an unpublished
 * entry before it gives up (0 restores the default, about a second of
 * waiting).  gsr_debug_stall_sort(1) makes the first digit pass of every
 * later sort leave its tile 0 untaken, so the tiles after it wait on an entry
 * that is never published; the sort then reports GSR_TIMEOUT through the
 * status word (gsr_read_status / gsr_sort_bits_static_status) and writes
 * nothing outside its buffers.  Both apply to sorts launched after the call. */
gsr_status gsr_debug_set_sort_wait_limit(uint32_t spins);
gsr_status gsr_debug_stall_sort(int on);

#ifdef __cplusplus
}
#endif

#endif /* GSR_H_ */
