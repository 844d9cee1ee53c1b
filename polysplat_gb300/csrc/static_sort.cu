// The pair sort backed by scratch the library owns: no allocation anywhere.
//
// Every other sort entry point takes a caller-provided workspace.  Some
// callers cannot provide one: a host that binds this library through a thin
// FFI and hands over only the key and value buffers (it has no allocator of
// its own for device memory), and latency-bound loops that must not call
// cudaMalloc, which can synchronise the whole device and stall other work.
// This entry sorts up to kStaticSortKeys pairs in a file-scope device array
// instead.  That array is shared by every call in the process, so calls that
// overlap in time (on different streams or from different host threads) race
// on it and must be serialised by the caller.  A bounded wait that runs out
// inside such a sort is recorded in the array's status word, which
// gsr_sort_bits_static_status() reads back.
//
// The array's device address is looked up once per device and kept for the
// life of the process; after cudaDeviceReset() on a device this entry point
// must not be called on that device again.
#include <mutex>

#include "gsr_internal.h"

namespace gsr {
namespace {

constexpr long long kStaticSortKeys = 1LL << 18;  // 262,144 pairs
constexpr size_t align256s(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kStaticTiles = (size_t)((kStaticSortKeys + kSortTile - 1) / kSortTile);
// header (counters, histograms, status) + alternate keys and values + two
// look-back arrays: the layout carve_sort_scratch expects after the header
constexpr size_t kStaticScratchBytes = kHeaderBytes + align256s((size_t)kStaticSortKeys * 8) +
                                       align256s((size_t)kStaticSortKeys * 4) +
                                       2 * align256s(kStaticTiles * 256 * 4);

__device__ __align__(256) unsigned char g_static_sort_scratch[kStaticScratchBytes];

void* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mu;

// Address of the scratch array on the current device.  Looked up once per
// device (the first call on that device) and cached; nothing is allocated.
cudaError_t static_scratch(void** out)
{
    const int dev = current_device();
    if (dev < 0) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_sort_scratch);
        if (e != cudaSuccess) return e;
        if (!p) return cudaErrorInvalidSymbol;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

}  // namespace
}  // namespace gsr

using namespace gsr;

extern "C" gsr_status gsr_sort_bits_static(int num, const int32_t* d_num, int end_bit, const uint64_t* keys_in,
                                           const uint32_t* values_in, uint64_t* keys_out, uint32_t* values_out,
                                           int64_t capacity, gsr_stream_t stream)
{
    if (end_bit < 1 || end_bit > 64 || capacity < 0 || (!d_num && num < 0)) return GSR_INVALID_ARG;
    if (capacity > kStaticSortKeys) return GSR_INVALID_ARG;  // beyond the static scratch
    if (!d_num && num > capacity) return GSR_INVALID_ARG;
    if (capacity > 0 && (!keys_in || !values_in || !keys_out || !values_out)) return GSR_INVALID_ARG;
    if (keys_in == keys_out || values_in == values_out) return GSR_INVALID_ARG;
    void* base = nullptr;
    cudaError_t e = static_scratch(&base);
    if (e != cudaSuccess) return GSR_CUDA_ERROR;
    cudaStream_t s = (cudaStream_t)stream;
    WorkspaceHeader* hdr = reinterpret_cast<WorkspaceHeader*>(base);
    // the status word starts at zero; the sort clears its own counters and
    // histograms and the look-back arrays before it uses them
    e = cudaMemsetAsync(&hdr->status, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return GSR_CUDA_ERROR;
    const SortScratch sc = carve_sort_scratch(hdr, reinterpret_cast<char*>(base) + kHeaderBytes, kStaticSortKeys, 8);
    const OrderMap order{kOrderMasked, end_bit, 32};  // tile << 32 | depth bits
    e = launch_sort64(num, d_num, capacity, order, (end_bit + 7) / 8, keys_in, values_in, keys_out, values_out, sc, s);
    return e == cudaSuccess ? GSR_OK : (e == cudaErrorInvalidValue ? GSR_INVALID_ARG : GSR_CUDA_ERROR);
}

extern "C" gsr_status gsr_sort_bits_static_status(gsr_stream_t stream)
{
    // the status word is the first word of the array's header; read it on the
    // sort's stream, after the sort, into host memory (nothing is allocated)
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t status = 0;
    cudaError_t e = cudaMemcpyFromSymbolAsync(&status, g_static_sort_scratch, sizeof(status),
                                              offsetof(WorkspaceHeader, status), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return GSR_CUDA_ERROR;
    if (status & kErrTimeout) return GSR_TIMEOUT;
    if (status & kErrBadInput) return GSR_INVALID_ARG;
    return GSR_OK;
}
