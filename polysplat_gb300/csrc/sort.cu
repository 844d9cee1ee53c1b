// Stable LSD radix sort of (key, u32 value) pairs for sm_103a, for 64-bit
// tile|depth keys and for 32-bit keys.
//
// Contract of the 64-bit sort (the reference's CUB call,
// csrc/cuda_rasterizer/sort.cu:107-125): ascending, stable, unsigned, over
// bits [0, end_bit); bits at or above end_bit ride along but do not take part
// in the order; the inputs are preserved.  The count may live on the device,
// so no host synchronisation is needed between the producer and the sort.
//
// Structure (one-sweep radix sort with decoupled look-back):
//   1. k_upsweep: one read of all keys builds the 256-bin histogram of the
//      first 8-bit digit, and clears the first look-back array.
//   2. k_pass (one launch per digit): persistent CTAs take 4096-key tiles in
//      order from an atomic counter, rank keys stably inside the tile (per-warp
//      ranking by match.any or by bit ballots), publish per-digit tile counts,
//      look back over earlier tiles for the running per-digit prefix (bounded
//      spin, four predecessors per round trip), reorder the tile in shared
//      memory by digit and write it out with coalesced stores.  While it holds
//      a tile's keys it also counts their next digit, so the next pass's
//      histogram is complete when this launch ends.
//
// Keys are mapped to an "ordering word" before digits are taken (OrderMap):
// the masked key, or -- for keys the preprocess emitted -- the depth bits
// minus the bits of 0.2f, whose width the preprocess recorded in the
// workspace header.  When fewer bits matter than the host planned for, the
// remaining pass launches return at once, and every pass picks its source and
// destination buffer on the device so that the last working pass lands in the
// output.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>

#include "gsr_internal.h"

namespace gsr {
namespace {

constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
constexpr int kWarpsPerCta = kSortThreads / 32;
constexpr int kWarpItems = kSortItems * 32;  // consecutive keys per warp

template <typename K>
struct SortJob {
    int num;
    const int32_t* d_num;
    long long cap;
    OrderMap order;
    const K* keys_in;
    const uint32_t* vals_in;
    K* keys_out;
    uint32_t* vals_out;
    SortScratch s;
    uint32_t spin_limit;  // look-back spin bound (sort_wait_limit() at launch)
};

template <typename K>
__device__ __forceinline__ int sort_count(const SortJob<K>& a)
{
    long long n = a.d_num ? (long long)*a.d_num : (long long)a.num;
    if (n < 0) n = 0;
    if (n > a.cap) n = a.cap;
    return (int)n;
}

__host__ __device__ inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// The ordering word of a key and how many of its bits matter.
struct KeyMap {
    int kind;
    int bits;
    int depth_bits;
    uint64_t mask;
    uint32_t tile_mask;
};

__device__ __forceinline__ int depth_width(const WorkspaceHeader* h)
{
    const uint32_t hi = h->depth_hi;
    return hi > kDepthBitsFloor ? bits_for(hi - kDepthBitsFloor) : 0;
}

__device__ __forceinline__ KeyMap key_map(const OrderMap& o, const WorkspaceHeader* h)
{
    KeyMap m;
    m.kind = o.kind;
    m.depth_bits = 0;
    m.tile_mask = 0;
    m.bits = o.end_bit;
    m.mask = o.end_bit >= 64 ? ~0ull : ((1ull << o.end_bit) - 1ull);
    if (o.kind == kOrderDepthCompressed64) {
        m.depth_bits = depth_width(h);
        m.tile_mask = (uint32_t)((1ull << (o.end_bit - 32)) - 1ull);
        m.bits = (o.end_bit - 32) + m.depth_bits;
    } else if (o.kind == kOrderDepth32) {
        m.bits = depth_width(h);
    }
    if (m.bits < 1) m.bits = 1;
    return m;
}

__device__ __forceinline__ uint64_t order_word(uint64_t k, const KeyMap& m)
{
    if (m.kind == kOrderDepthCompressed64) {
        const uint64_t tile = (uint64_t)((uint32_t)(k >> 32) & m.tile_mask);
        return (tile << m.depth_bits) | (uint64_t)((uint32_t)k - kDepthBitsFloor);
    }
    return k & m.mask;
}

__device__ __forceinline__ uint64_t order_word(uint32_t k, const KeyMap& m)
{
    if (m.kind == kOrderDepth32) return (uint64_t)(k - kDepthBitsFloor);
    return (uint64_t)k & m.mask;
}

__device__ __forceinline__ int passes_of(const KeyMap& m) { return (m.bits + 7) / 8; }

// Eight consecutive keys from position b (a multiple of 8): 16-byte loads
// for a full run of a 16-byte aligned buffer, single loads otherwise.
template <typename K>
__device__ __forceinline__ void load8(const K* src, long long b, int cnt, K (&k)[8])
{
    if (cnt == 8 && (reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
        constexpr int kPer = 16 / sizeof(K);
        const uint4* v = reinterpret_cast<const uint4*>(src + b);
#pragma unroll
        for (int q = 0; q < 8 / kPer; q++) {
            const uint4 w = __ldg(v + q);
            const K* e = reinterpret_cast<const K*>(&w);
#pragma unroll
            for (int j = 0; j < kPer; j++) k[q * kPer + j] = e[j];
        }
        return;
    }
#pragma unroll
    for (int j = 0; j < 8; j++) k[j] = j < cnt ? __ldg(src + b + j) : K(0);
}

// ---------------------------------------------------------------------------
// Histogram of the first digit pass; every digit pass counts the next one's
// digits from the keys it holds anyway (one read of the keys instead of one
// per pass here: 27 against 44 us at 9.2 M keys).  Each thread takes runs of
// 8 consecutive keys and merges equal consecutive digits before touching
// shared memory: keys of one Gaussian are emitted together and share their
// depth digits, so this removes most same-address shared atomics.
template <typename K>
__global__ __launch_bounds__(256) void k_upsweep(SortJob<K> a)
{
    __shared__ uint32_t s_hist[256];
    s_hist[threadIdx.x] = 0u;
    __syncthreads();
    const int n = sort_count(a);
    const int tiles = (n + kSortTile - 1) / kSortTile;
    const KeyMap km = key_map(a.order, a.s.hdr);
    // clear the look-back state used by the first digit pass
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)tiles * 256;
         i += (long long)gridDim.x * blockDim.x)
        a.s.look[0][i] = 0u;

    const long long runs = (n + 7) / 8;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < runs;
         r += (long long)gridDim.x * blockDim.x) {
        const long long b = r * 8;
        K kk[8];
        const int cnt = (int)min(8LL, (long long)n - b);
        load8(a.keys_in, b, cnt, kk);
        uint32_t cur = (uint32_t)order_word(kk[0], km) & 0xFFu;
        uint32_t run = 1;
#pragma unroll
        for (int j = 1; j < 8; j++) {
            if (j >= cnt) break;
            const uint32_t d = (uint32_t)order_word(kk[j], km) & 0xFFu;
            if (d == cur) {
                run++;
            } else {
                atomicAdd(&s_hist[cur], run);
                cur = d;
                run = 1;
            }
        }
        atomicAdd(&s_hist[cur], run);
    }
    __syncthreads();
    if (s_hist[threadIdx.x]) atomicAdd(&a.s.hdr->hist[0][threadIdx.x], s_hist[threadIdx.x]);
}

// ---------------------------------------------------------------------------
template <typename K>
struct PassSmem {
    K keys[kSortTile];
    uint32_t vals[kSortTile];
    uint8_t digs[kSortTile];            // each reordered key's digit, so the scatter need not recompute it
    uint32_t whist[kWarpsPerCta][256];  // per-warp digit counts, then warp-exclusive offsets
    uint32_t digit_excl[256];           // tile-local start of each digit
    int gofs[256];                      // global position of tile position 0 per digit
    uint32_t gstart[256];               // global start of each digit (scan of histogram)
    uint32_t next_hist[256];            // this CTA's counts of the next pass's digit
    uint32_t warp_sums[kWarpsPerCta];
    int tile;
};

// Exclusive scan of one value per thread over the whole CTA (kSortThreads);
// the digit passes hold digit d's value in thread d and zeros above 255.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* warp_sums)
{
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t n = __shfl_up_sync(GSR_FULL_MASK, incl, d);
        if (lane >= (unsigned)d) incl += n;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    uint32_t wpre = 0;
#pragma unroll
    for (int w = 0; w < kWarpsPerCta; w++)
        if (w < (int)warp) wpre += warp_sums[w];
    __syncthreads();
    return wpre + incl - v;
}

// One digit pass.  Keys are ranked within each warp either with match.any
// (one instruction per key) or with one ballot per digit bit.  RANK 2 picks
// per pass: match.any for depth digits, ballots for digits holding tile ids
// (measured at 3 M Gaussians / 1080p: 93 vs 111 us on depth digits, 134 vs
// 120 us and 125 vs 109 us on the two tile-bit passes); RANK 0 / 1 force
// ballots / match.any.
template <typename K, int RANK>
__global__ __launch_bounds__(kSortThreads, 2) void k_pass(SortJob<K> a, int pass)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PassSmem<K>& S = *reinterpret_cast<PassSmem<K>*>(smem_raw);
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const KeyMap km = key_map(a.order, a.s.hdr);
    const int passes = passes_of(km);
    if (pass >= passes) return;  // nothing left to order in this digit
    const int n = sort_count(a);
    const int tiles = (n + kSortTile - 1) / kSortTile;
    const int shift = 8 * pass;
    const int bits = min(8, km.bits - shift);
    const int tile_from = a.order.kind == kOrderDepthCompressed64 ? km.depth_bits : a.order.tile_from_bit;
    const bool use_match = RANK == 1 || (RANK == 2 && shift + bits <= tile_from);
    // ping-pong so that the last working pass writes the output buffers
    const bool to_out = ((passes - 1 - pass) & 1) == 0;
    K* alt_k = reinterpret_cast<K*>(a.s.alt_keys);
    const K* kin = a.keys_in;
    const uint32_t* vin = a.vals_in;
    if (pass > 0) {
        const bool prev_out = ((passes - pass) & 1) == 0;
        kin = prev_out ? a.keys_out : alt_k;
        vin = prev_out ? a.vals_out : a.s.alt_vals;
    }
    K* kout = to_out ? a.keys_out : alt_k;
    uint32_t* vout = to_out ? a.vals_out : a.s.alt_vals;
    // selects rather than a dynamic index, so the parameter block stays out of local memory
    uint32_t* look = (pass & 1) ? a.s.look[1] : a.s.look[0];
    uint32_t* look_next = (pass & 1) ? a.s.look[0] : a.s.look[1];
    const bool clear_next = pass + 1 < passes;
    WorkspaceHeader* hdr = a.s.hdr;

    const bool digit_thread = threadIdx.x < 256;  // thread d owns digit d in the per-digit steps
    // the next pass's histogram is counted here, from the keys this pass holds
    const bool count_next = pass + 1 < passes;
    if (digit_thread) S.next_hist[threadIdx.x] = 0u;
    {
        const uint32_t g = block_excl_scan(digit_thread ? hdr->hist[pass][threadIdx.x] : 0u, S.warp_sums);
        if (digit_thread) S.gstart[threadIdx.x] = g;
    }

    for (;;) {
        if (threadIdx.x == 0) S.tile = (int)atomicAdd(&hdr->pass_counter[pass], 1u);
        for (int i = threadIdx.x; i < kWarpsPerCta * 256; i += kSortThreads) (&S.whist[0][0])[i] = 0u;
        __syncthreads();
        const int tile = S.tile;
        if (tile >= tiles) break;
        const long long tbase = (long long)tile * kSortTile;
        const int tcount = (int)min((long long)kSortTile, (long long)n - tbase);
        if (clear_next && digit_thread) look_next[(size_t)tile * 256 + threadIdx.x] = 0u;

        // ---- load (warp-contiguous chunk) + stable per-warp rank ----
        K key[kSortItems];
        uint32_t val[kSortItems];
        uint32_t dig[kSortItems];
        uint32_t rank[kSortItems];
        const int wbase = (int)warp * kWarpItems;
#pragma unroll
        for (int i = 0; i < kSortItems; i++) {
            const int o = wbase + i * 32 + (int)lane;
            if (o < tcount) {
                key[i] = kin[tbase + o];
                val[i] = vin[tbase + o];
            } else {
                key[i] = K(0);
                val[i] = 0u;
            }
        }
#pragma unroll
        for (int i = 0; i < kSortItems; i++) {
            const int o = wbase + i * 32 + (int)lane;
            const bool ok = o < tcount;
            const uint64_t w = order_word(key[i], km);
            const uint32_t d = (uint32_t)(w >> shift) & ((1u << bits) - 1u);
            dig[i] = d;
            if (count_next && ok) atomicAdd(&S.next_hist[(uint32_t)(w >> (shift + 8)) & 0xFFu], 1u);
            if (use_match) {
                // out-of-range lanes get a value no real digit has
                const unsigned peers = __match_any_sync(GSR_FULL_MASK, ok ? d : 0x100u + lane);
                const int leader = __ffs(peers) - 1;
                uint32_t base = 0;
                if (ok && (int)lane == leader) {
                    base = S.whist[warp][d];
                    S.whist[warp][d] = base + __popc(peers);
                }
                base = __shfl_sync(GSR_FULL_MASK, base, leader);
                rank[i] = base + __popc(peers & lanemask_lt());
            } else {
                unsigned peers = __ballot_sync(GSR_FULL_MASK, ok);
                for (int b = 0; b < bits; b++) {
                    const bool bit = (d >> b) & 1u;
                    const unsigned bb = __ballot_sync(GSR_FULL_MASK, bit);
                    peers &= bit ? bb : ~bb;
                }
                uint32_t base = 0;
                if (ok) base = S.whist[warp][d];
                __syncwarp();
                if (ok && (lane == (unsigned)(__ffs(peers) - 1))) S.whist[warp][d] = base + __popc(peers);
                __syncwarp();
                rank[i] = base + __popc(peers & lanemask_lt());
            }
        }
        __syncthreads();

        // ---- per-digit offsets across warps; publish the tile's counts;
        //      offsets across digits ----
        uint32_t dtot = 0;
        {
            const int d = threadIdx.x;
            if (digit_thread) {
#pragma unroll
                for (int w = 0; w < kWarpsPerCta; w++) {
                    uint32_t c = S.whist[w][d];
                    S.whist[w][d] = dtot;
                    dtot += c;
                }
                // later tiles' look-back can use the count before this tile's scan is done
                st_relaxed_u32(look + (size_t)tile * 256 + d, (tile == 0 ? kFlagPrefix : kFlagAgg) | dtot);
            }
            const uint32_t ex = block_excl_scan(dtot, S.warp_sums);
            if (digit_thread) S.digit_excl[d] = ex;
        }
        __syncthreads();  // digit_excl complete

        // ---- reorder in shared memory: the warps without a digit do it while
        //      the digit warps look back, and the digit warps after ----
        auto reorder = [&]() {
#pragma unroll
            for (int i = 0; i < kSortItems; i++) {
                const int o = wbase + i * 32 + (int)lane;
                if (o < tcount) {
                    const uint32_t pos = S.digit_excl[dig[i]] + S.whist[warp][dig[i]] + rank[i];
                    S.keys[pos] = key[i];
                    S.vals[pos] = val[i];
                    S.digs[pos] = (uint8_t)dig[i];
                }
            }
        };
        if (!digit_thread) reorder();

        // ---- decoupled look-back: thread d owns digit d ----
        if (digit_thread) {
            const int d = threadIdx.x;
            uint32_t* my = look + (size_t)tile * 256 + d;
            // walk back four predecessors per round trip; stop at the first
            // inclusive prefix, re-reading any entry that is not published yet
            uint32_t excl = 0;
            int j = tile - 1;
            uint32_t spins = 0;
            bool done = j < 0;
            while (!done) {
                // four predecessors per round trip: measured faster than 8
                // (+6%) or 16 (+25%) at 9.2 M keys
                uint32_t v[4];
#pragma unroll
                for (int k = 0; k < 4; k++)
                    v[k] = (j - k >= 0) ? ld_relaxed_u32(look + (size_t)(j - k) * 256 + d) : kFlagPrefix;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    if (done) break;
                    if ((v[k] & ~kValueMask) == 0u) break;  // not published yet: re-read from j
                    excl += v[k] & kValueMask;
                    j--;
                    if ((v[k] & kFlagPrefix) || j < 0) done = true;
                }
                if (!done && (v[0] & ~kValueMask) == 0u) {
                    if (++spins > a.spin_limit) {
                        record_error(&hdr->status, kErrTimeout);
                        break;
                    }
                    __nanosleep(32);
                }
            }
            if (tile != 0) st_relaxed_u32(my, kFlagPrefix | ((excl + dtot) & kValueMask));
            S.gofs[d] = (int)(S.gstart[d] + excl) - (int)S.digit_excl[d];
            reorder();
        }
        __syncthreads();

        // ---- coalesced scatter of the digit runs ----
        bool oob = false;
        for (int p = threadIdx.x; p < tcount; p += kSortThreads) {
            const K k = S.keys[p];
            const long long g = (long long)S.gofs[S.digs[p]] + p;
            if (g < 0 || g >= n) {  // only after a look-back timeout: never write outside the buffer
                oob = true;
                continue;
            }
            kout[g] = k;
            vout[g] = S.vals[p];
        }
        if (oob) record_error(&hdr->status, kErrTimeout);
        __syncthreads();
    }
    // every count of this CTA precedes the barrier that ended its last tile
    if (count_next && digit_thread && S.next_hist[threadIdx.x])
        atomicAdd(&hdr->hist[pass + 1][threadIdx.x], S.next_hist[threadIdx.x]);
}

// 2 (choose per sort and pass) unless GSR_SORT_RANK asks for "ballot" (0) or
// "match" (1) everywhere
int sort_rank_mode()
{
    static const int mode = [] {  // read once, thread-safe initialisation
        const char* e = getenv("GSR_SORT_RANK");
        return (e && strcmp(e, "ballot") == 0) ? 0 : (e && strcmp(e, "match") == 0) ? 1 : 2;
    }();
    return mode;
}

template <typename K>
cudaError_t run_sort(const SortJob<K>& job, int max_passes, cudaStream_t stream)
{
    if (job.cap >= (1LL << 30) || max_passes < 1 || max_passes > kMaxPasses) return cudaErrorInvalidValue;
    SortJob<K> a = job;
    a.spin_limit = sort_wait_limit();
    // clear the sort region of the header (pass counters and histograms)
    cudaError_t e = cudaMemsetAsync(reinterpret_cast<char*>(a.s.hdr) + kSortRegionOffset, 0,
                                    sizeof(WorkspaceHeader) - kSortRegionOffset, stream);
    if (e != cudaSuccess) return e;
    // failure-detection hook: the first pass starts at tile 1, so tile 0 never
    // publishes and the look-back of the tiles after it runs out
    if (sort_stall_first_tile() && (e = cudaMemsetAsync(&a.s.hdr->pass_counter[0], 1, 1, stream)) != cudaSuccess)
        return e;
    const int sms = device_sm_count();
    int up_grid = (int)std::min<long long>((long long)sms * 4, std::max<long long>(1, (a.cap + 2047) / 2048));
    k_upsweep<K><<<up_grid, 256, 0, stream>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    profile_mark(stream);

    // per-pass choice only where depth and tile digits share the key; the
    // choice costs a uniform branch per key, so all-depth and all-tile sorts
    // keep the branch-free match.any kernel
    const bool mixed = a.order.kind == kOrderDepthCompressed64 ||
                       (a.order.tile_from_bit > 0 && a.order.tile_from_bit < a.order.end_bit);
    const int forced = sort_rank_mode();
    const int mode = forced != 2 ? forced : (mixed ? 2 : 1);
    auto kern = mode == 0 ? k_pass<K, 0> : mode == 1 ? k_pass<K, 1> : k_pass<K, 2>;
    // per device and ranking mode: the shared-memory attribute (a property of
    // the kernel on each device), then the occupancy; host threads may race
    // to fill these with the same values
    static std::atomic<int> per_sm_cache[kMaxDevices][3];
    const int dev = current_device();
    if (dev < 0) return cudaErrorInvalidDevice;
    const int smem = (int)sizeof(PassSmem<K>);
    int per_sm = per_sm_cache[dev][mode].load(std::memory_order_acquire);
    if (per_sm == 0) {
        if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess)
            return e;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSortThreads, smem) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        per_sm_cache[dev][mode].store(per_sm, std::memory_order_release);
    }
    const int grid = (int)std::min<long long>((long long)sms * per_sm, std::max<long long>(1, a.s.tiles_cap));
    for (int p = 0; p < max_passes; p++) {
        kern<<<grid, kSortThreads, smem, stream>>>(a, p);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        profile_mark(stream);
    }
    return cudaSuccess;
}

}  // namespace

// ---------------------------------------------------------------------------
// Workspace layout: [header+queue][alt keys 8*cap][alt vals 4*cap][look-back x2][tile ranges]

static size_t sort_area_bytes(long long cap)
{
    if (cap < 1) cap = 1;
    long long tiles = (cap + kSortTile - 1) / kSortTile;
    return kSmallWorkspaceBytes + align256((size_t)cap * 8) + align256((size_t)cap * 4) +
           2 * align256((size_t)tiles * 256 * 4);
}

size_t sort_workspace_bytes(long long cap) { return sort_area_bytes(cap) + (size_t)kWorkspaceRangeTiles * 8; }

int2* workspace_ranges(void* ws, long long cap)
{
    return reinterpret_cast<int2*>(reinterpret_cast<char*>(ws) + sort_area_bytes(cap));
}

SortScratch workspace_sort_scratch(void* ws, long long cap)
{
    SortScratch s;
    char* p = reinterpret_cast<char*>(ws);
    s.hdr = reinterpret_cast<WorkspaceHeader*>(p);
    size_t off = kSmallWorkspaceBytes;
    s.alt_keys = p + off;
    off += align256((size_t)(cap < 1 ? 1 : cap) * 8);
    s.alt_vals = reinterpret_cast<uint32_t*>(p + off);
    off += align256((size_t)(cap < 1 ? 1 : cap) * 4);
    s.tiles_cap = ((cap < 1 ? 1 : cap) + kSortTile - 1) / kSortTile;
    s.look[0] = reinterpret_cast<uint32_t*>(p + off);
    off += align256((size_t)s.tiles_cap * 256 * 4);
    s.look[1] = reinterpret_cast<uint32_t*>(p + off);
    return s;
}

size_t sort_scratch_bytes(long long cap, int key_bytes)
{
    if (cap < 1) cap = 1;
    long long tiles = (cap + kSortTile - 1) / kSortTile;
    return align256((size_t)cap * key_bytes) + align256((size_t)cap * 4) + 2 * align256((size_t)tiles * 256 * 4);
}

SortScratch carve_sort_scratch(WorkspaceHeader* hdr, void* mem, long long cap, int key_bytes)
{
    SortScratch s;
    char* p = reinterpret_cast<char*>(mem);
    s.hdr = hdr;
    if (cap < 1) cap = 1;
    s.alt_keys = p;
    size_t off = align256((size_t)cap * key_bytes);
    s.alt_vals = reinterpret_cast<uint32_t*>(p + off);
    off += align256((size_t)cap * 4);
    s.tiles_cap = (cap + kSortTile - 1) / kSortTile;
    s.look[0] = reinterpret_cast<uint32_t*>(p + off);
    off += align256((size_t)s.tiles_cap * 256 * 4);
    s.look[1] = reinterpret_cast<uint32_t*>(p + off);
    return s;
}

cudaError_t launch_sort(const SortArgs& a, cudaStream_t stream)
{
    if (a.end_bit < 1 || a.end_bit > 64) return cudaErrorInvalidValue;
    if (a.ws_bytes < sort_area_bytes(a.cap)) return cudaErrorInvalidValue;
    SortJob<uint64_t> j;
    j.num = a.num;
    j.d_num = a.d_num;
    j.cap = a.cap;
    j.order.kind = a.compress_depth && a.end_bit > 32 ? kOrderDepthCompressed64 : kOrderMasked;
    j.order.end_bit = a.end_bit;
    j.order.tile_from_bit = 32;  // tile << 32 | depth bits
    j.keys_in = a.keys_in;
    j.vals_in = a.vals_in;
    j.keys_out = a.keys_out;
    j.vals_out = a.vals_out;
    j.s = workspace_sort_scratch(a.ws, a.cap);
    j.spin_limit = kSpinLimit;
    return run_sort(j, (a.end_bit + 7) / 8, stream);
}

cudaError_t launch_sort32(int num, const int32_t* d_num, long long cap, OrderMap order, int max_passes,
                          const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                          const SortScratch& s, cudaStream_t stream)
{
    SortJob<uint32_t> j;
    j.num = num;
    j.d_num = d_num;
    j.cap = cap;
    j.order = order;
    j.keys_in = keys_in;
    j.vals_in = vals_in;
    j.keys_out = keys_out;
    j.vals_out = vals_out;
    j.s = s;
    j.spin_limit = kSpinLimit;
    return run_sort(j, max_passes, stream);
}

cudaError_t launch_sort64(int num, const int32_t* d_num, long long cap, OrderMap order, int max_passes,
                          const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out, uint32_t* vals_out,
                          const SortScratch& s, cudaStream_t stream)
{
    SortJob<uint64_t> j;
    j.num = num;
    j.d_num = d_num;
    j.cap = cap;
    j.order = order;
    j.keys_in = keys_in;
    j.vals_in = vals_in;
    j.keys_out = keys_out;
    j.vals_out = vals_out;
    j.s = s;
    j.spin_limit = kSpinLimit;
    return run_sort(j, max_passes, stream);
}

}  // namespace gsr
