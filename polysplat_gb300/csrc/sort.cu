// Stable LSD radix sort of (u64 key, u32 value) pairs for sm_103a.
//
// Contract (same as the reference's CUB call, csrc/cuda_rasterizer/sort.cu:
// 107-125): ascending, stable, unsigned, over bits [0, end_bit); bits at or
// above end_bit ride along but do not take part in the order; the inputs are
// preserved.  The count may live on the device, so no host synchronisation
// is needed between the producer of the keys and the sort.
//
// Structure (one-sweep radix sort with decoupled look-back):
//   1. k_upsweep: one read of all keys builds the 256-bin histogram of every
//      8-bit digit pass at once, and clears the first look-back array.
//   2. k_pass (one launch per digit): persistent CTAs take 2048-key tiles in
//      order from an atomic counter, rank keys stably inside the tile (per-warp
//      ranking by match.any or by bit ballots), publish per-digit tile counts,
//      look back over earlier tiles for the running per-digit prefix (bounded
//      spin, four predecessors per round trip), reorder the tile in shared
//      memory by digit and write it out with coalesced stores.
//
// Depth compression (fused forward): every emitted key has a low word above
// the bits of 0.2f and at most the header's depth_hi, so ordering by
// (tile << nb) | (low - floor) with nb = bits(depth_hi - floor) is the same
// order in fewer bits.  The number of passes that do work is then decided on
// the device; the remaining launches return at once, and each pass picks its
// source and destination buffer so that the last working pass lands in the
// output.
#include <algorithm>
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

__device__ __forceinline__ int sort_count(const SortArgs& a)
{
    long long n = a.d_num ? (long long)*a.d_num : (long long)a.num;
    if (n < 0) n = 0;
    if (n > a.cap) n = a.cap;
    return (int)n;
}

struct Layout {
    WorkspaceHeader* hdr;
    uint64_t* alt_keys;
    uint32_t* alt_vals;
    uint32_t* look[2];
    long long tiles_cap;
};

__host__ __device__ inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

__host__ __device__ inline Layout make_layout(void* ws, long long cap)
{
    Layout L;
    char* p = reinterpret_cast<char*>(ws);
    L.hdr = reinterpret_cast<WorkspaceHeader*>(p);
    size_t off = kSmallWorkspaceBytes;  // header + massive-Gaussian queue
    L.alt_keys = reinterpret_cast<uint64_t*>(p + off);
    off += align256((size_t)cap * 8);
    L.alt_vals = reinterpret_cast<uint32_t*>(p + off);
    off += align256((size_t)cap * 4);
    L.tiles_cap = (cap + kSortTile - 1) / kSortTile;
    L.look[0] = reinterpret_cast<uint32_t*>(p + off);
    off += align256((size_t)L.tiles_cap * 256 * 4);
    L.look[1] = reinterpret_cast<uint32_t*>(p + off);
    return L;
}

// The ordering word of a key and the number of its bits that matter.
struct KeyMap {
    int bits;           // significant bits of the ordering word
    int depth_bits;     // 0: no compression
    uint64_t mask;      // mask of the uncompressed key (end_bit bits)
    uint32_t tile_mask;
};

__device__ __forceinline__ KeyMap key_map(const SortArgs& a, const Layout& L)
{
    KeyMap m;
    m.mask = a.end_bit >= 64 ? ~0ull : ((1ull << a.end_bit) - 1ull);
    m.depth_bits = 0;
    m.tile_mask = 0;
    m.bits = a.end_bit;
    if (a.compress_depth && a.end_bit > 32) {
        const uint32_t hi = L.hdr->depth_hi;
        const int nb = hi > kDepthBitsFloor ? bits_for(hi - kDepthBitsFloor) : 0;
        m.depth_bits = nb;
        m.tile_mask = (uint32_t)((1ull << (a.end_bit - 32)) - 1ull);
        m.bits = (a.end_bit - 32) + nb;
        if (m.bits < 1) m.bits = 1;
    }
    return m;
}

__device__ __forceinline__ uint64_t order_word(uint64_t k, const KeyMap& m)
{
    if (m.tile_mask == 0) return k & m.mask;
    const uint64_t tile = (uint64_t)((uint32_t)(k >> 32) & m.tile_mask);
    return (tile << m.depth_bits) | (uint64_t)((uint32_t)k - kDepthBitsFloor);
}

__device__ __forceinline__ int passes_of(const KeyMap& m) { return (m.bits + 7) / 8; }

// ---------------------------------------------------------------------------
// Histogram of every digit pass.  Each thread takes runs of 8 consecutive keys
// and merges equal consecutive digits before touching shared memory: keys of
// one Gaussian are emitted together and share their depth digits, so this
// removes most same-address shared atomics.
__global__ __launch_bounds__(256) void k_upsweep(SortArgs a, Layout L, int max_passes)
{
    __shared__ uint32_t s_hist[kMaxPasses][256];
    for (int i = threadIdx.x; i < kMaxPasses * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0u;
    __syncthreads();
    const int n = sort_count(a);
    const int tiles = (n + kSortTile - 1) / kSortTile;
    const KeyMap km = key_map(a, L);
    const int passes = min(max_passes, passes_of(km));
    // clear the look-back state used by the first digit pass
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)tiles * 256;
         i += (long long)gridDim.x * blockDim.x)
        L.look[0][i] = 0u;

    const long long runs = (n + 7) / 8;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < runs;
         r += (long long)gridDim.x * blockDim.x) {
        const long long b = r * 8;
        uint64_t k[8];
        const int cnt = (int)min(8LL, (long long)n - b);
        if (cnt == 8 && ((reinterpret_cast<uintptr_t>(a.keys_in + b) & 15) == 0)) {
            const uint4* src = reinterpret_cast<const uint4*>(a.keys_in + b);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                uint4 v = __ldg(src + j);
                k[2 * j] = ((uint64_t)v.y << 32) | v.x;
                k[2 * j + 1] = ((uint64_t)v.w << 32) | v.z;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 8; j++) k[j] = j < cnt ? __ldg(a.keys_in + b + j) : 0ull;
        }
#pragma unroll
        for (int j = 0; j < 8; j++) k[j] = order_word(k[j], km);
        for (int p = 0; p < passes; p++) {
            const int shift = 8 * p;
            uint32_t cur = (uint32_t)(k[0] >> shift) & 0xFFu;
            uint32_t run = 1;
#pragma unroll
            for (int j = 1; j < 8; j++) {
                if (j >= cnt) break;
                uint32_t d = (uint32_t)(k[j] >> shift) & 0xFFu;
                if (d == cur) {
                    run++;
                } else {
                    atomicAdd(&s_hist[p][cur], run);
                    cur = d;
                    run = 1;
                }
            }
            atomicAdd(&s_hist[p][cur], run);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        uint32_t v = (&s_hist[0][0])[i];
        if (v) atomicAdd(&L.hdr->hist[0][0] + i, v);
    }
}

// ---------------------------------------------------------------------------
struct PassSmem {
    uint64_t keys[kSortTile];
    uint32_t vals[kSortTile];
    uint32_t whist[kWarpsPerCta][256];  // per-warp digit counts, then warp-exclusive offsets
    uint32_t digit_excl[256];           // tile-local start of each digit
    int gofs[256];                      // global position of tile position 0 per digit
    uint32_t gstart[256];               // global start of each digit (scan of histogram)
    uint32_t warp_sums[kWarpsPerCta];
    int tile;
};

// Exclusive scan of 256 values held one per thread (blockDim == 256).
__device__ __forceinline__ uint32_t block_excl_scan256(uint32_t v, uint32_t* warp_sums)
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

struct PassBuffers {
    const uint64_t* keys_in;
    const uint32_t* vals_in;
    uint64_t* keys_out;
    uint32_t* vals_out;
    uint64_t* keys_alt;
    uint32_t* vals_alt;
};

// MATCH: per-warp ranking with match.any (one instruction per key);
// otherwise with one ballot per digit bit.
template <bool MATCH>
__global__ __launch_bounds__(kSortThreads, 4) void k_pass(SortArgs a, Layout L, int pass, PassBuffers B)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PassSmem& S = *reinterpret_cast<PassSmem*>(smem_raw);
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const KeyMap km = key_map(a, L);
    const int passes = passes_of(km);
    if (pass >= passes) return;  // nothing left to order in this digit
    const int n = sort_count(a);
    const int tiles = (n + kSortTile - 1) / kSortTile;
    const int shift = 8 * pass;
    const int bits = min(8, km.bits - shift);
    // ping-pong so that the last working pass writes the output buffers
    const bool to_out = ((passes - 1 - pass) & 1) == 0;
    const uint64_t* kin = B.keys_in;
    const uint32_t* vin = B.vals_in;
    if (pass > 0) {
        const bool prev_out = ((passes - pass) & 1) == 0;
        kin = prev_out ? B.keys_out : B.keys_alt;
        vin = prev_out ? B.vals_out : B.vals_alt;
    }
    uint64_t* kout = to_out ? B.keys_out : B.keys_alt;
    uint32_t* vout = to_out ? B.vals_out : B.vals_alt;
    uint32_t* look = L.look[pass & 1];
    uint32_t* look_next = L.look[(pass + 1) & 1];
    const bool clear_next = pass + 1 < passes;

    S.gstart[threadIdx.x] = block_excl_scan256(L.hdr->hist[pass][threadIdx.x], S.warp_sums);

    for (;;) {
        if (threadIdx.x == 0) S.tile = (int)atomicAdd(&L.hdr->pass_counter[pass], 1u);
        for (int i = threadIdx.x; i < kWarpsPerCta * 256; i += kSortThreads) (&S.whist[0][0])[i] = 0u;
        __syncthreads();
        const int tile = S.tile;
        if (tile >= tiles) break;
        const long long tbase = (long long)tile * kSortTile;
        const int tcount = (int)min((long long)kSortTile, (long long)n - tbase);
        if (clear_next) look_next[(size_t)tile * 256 + threadIdx.x] = 0u;

        // ---- load (warp-contiguous chunk) + stable per-warp rank ----
        uint64_t key[kSortItems];
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
                key[i] = 0ull;
                val[i] = 0u;
            }
        }
#pragma unroll
        for (int i = 0; i < kSortItems; i++) {
            const int o = wbase + i * 32 + (int)lane;
            const bool ok = o < tcount;
            const uint32_t d = (uint32_t)(order_word(key[i], km) >> shift) & ((1u << bits) - 1u);
            dig[i] = d;
            if (MATCH) {
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

        // ---- per-digit offsets: across warps, then across digits ----
        uint32_t dtot;
        {
            const int d = threadIdx.x;
            uint32_t run = 0;
#pragma unroll
            for (int w = 0; w < kWarpsPerCta; w++) {
                uint32_t c = S.whist[w][d];
                S.whist[w][d] = run;
                run += c;
            }
            dtot = run;
            S.digit_excl[d] = block_excl_scan256(run, S.warp_sums);
        }

        // ---- decoupled look-back: thread d owns digit d ----
        {
            const int d = threadIdx.x;
            uint32_t* my = look + (size_t)tile * 256 + d;
            st_relaxed_u32(my, (tile == 0 ? kFlagPrefix : kFlagAgg) | dtot);
            // walk back four predecessors per round trip; stop at the first
            // inclusive prefix, re-reading any entry that is not published yet
            uint32_t excl = 0;
            int j = tile - 1;
            uint32_t spins = 0;
            bool done = j < 0;
            while (!done) {
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
                    if (++spins > kSpinLimit) {
                        record_error(&L.hdr->status, kErrTimeout);
                        break;
                    }
                    __nanosleep(32);
                }
            }
            if (tile != 0) st_relaxed_u32(my, kFlagPrefix | ((excl + dtot) & kValueMask));
            S.gofs[d] = (int)(S.gstart[d] + excl) - (int)S.digit_excl[d];
        }
        __syncthreads();

        // ---- reorder in shared memory, then coalesced scatter ----
#pragma unroll
        for (int i = 0; i < kSortItems; i++) {
            const int o = wbase + i * 32 + (int)lane;
            if (o < tcount) {
                const uint32_t pos = S.digit_excl[dig[i]] + S.whist[warp][dig[i]] + rank[i];
                S.keys[pos] = key[i];
                S.vals[pos] = val[i];
            }
        }
        __syncthreads();
        bool oob = false;
        for (int p = threadIdx.x; p < tcount; p += kSortThreads) {
            const uint64_t k = S.keys[p];
            const uint32_t d = (uint32_t)(order_word(k, km) >> shift) & ((1u << bits) - 1u);
            const long long g = (long long)S.gofs[d] + p;
            if (g < 0 || g >= n) {  // only after a look-back timeout: never write outside the buffer
                oob = true;
                continue;
            }
            kout[g] = k;
            vout[g] = S.vals[p];
        }
        if (oob) record_error(&L.hdr->status, kErrTimeout);
        __syncthreads();
    }
}

bool use_match_ranking()
{
    static int mode = -1;
    if (mode < 0) {
        const char* e = getenv("GSR_SORT_RANK");
        mode = (e && strcmp(e, "ballot") == 0) ? 0 : 1;
    }
    return mode == 1;
}

}  // namespace

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

cudaError_t launch_sort(const SortArgs& a, cudaStream_t stream)
{
    if (a.end_bit < 1 || a.end_bit > 64) return cudaErrorInvalidValue;
    if (a.ws_bytes < sort_area_bytes(a.cap)) return cudaErrorInvalidValue;
    if (a.cap >= (1LL << 30)) return cudaErrorInvalidValue;
    Layout L = make_layout(a.ws, a.cap);
    const int passes = (a.end_bit + 7) / 8;  // upper bound; the device may need fewer
    // clear the sort region of the header (pass counters and histograms)
    cudaError_t e = cudaMemsetAsync(reinterpret_cast<char*>(L.hdr) + kSortRegionOffset, 0,
                                    sizeof(WorkspaceHeader) - kSortRegionOffset, stream);
    if (e != cudaSuccess) return e;
    const int sms = device_sm_count();
    const long long tiles_cap = L.tiles_cap;
    int up_grid = (int)std::min<long long>((long long)sms * 4, std::max<long long>(1, (a.cap + 2047) / 2048));
    k_upsweep<<<up_grid, 256, 0, stream>>>(a, L, passes);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    profile_mark(stream);

    const bool match = use_match_ranking();
    auto kern = match ? k_pass<true> : k_pass<false>;
    static bool attr_set[2] = {false, false};
    const int smem = (int)sizeof(PassSmem);
    if (!attr_set[match]) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr_set[match] = true;
    }
    static int per_sm[2] = {0, 0};
    if (per_sm[match] == 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, kSortThreads, smem) != cudaSuccess || b < 1) b = 1;
        per_sm[match] = b;
    }
    const int grid = (int)std::min<long long>((long long)sms * per_sm[match], std::max<long long>(1, tiles_cap));
    PassBuffers B{a.keys_in, a.vals_in, a.keys_out, a.vals_out, L.alt_keys, L.alt_vals};
    for (int p = 0; p < passes; p++) {
        kern<<<grid, kSortThreads, smem, stream>>>(a, L, p, B);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        profile_mark(stream);
    }
    return cudaSuccess;
}

}  // namespace gsr
