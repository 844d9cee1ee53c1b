// Launcher for the reference rasterizer's own CUDA kernels -- TEST INFRASTRUCTURE.
//
// oracle/ref_build.py compiles the reference's csrc/cuda_rasterizer/
// preprocess.cu and render.cu (unmodified, with the reference's nvcc flags)
// into cubins under oracle/_ref/.  This file loads those cubins with the CUDA
// driver API and launches the kernels exactly as the reference's host
// launchers do (grid/block shapes, argument lists), so the tests and the
// benchmark can compare this library with the reference's own GPU code on
// the same GB300:
//   preprocessCUDA            csrc/cuda_rasterizer/preprocess.cu:313, launch :1268-1329
//   computeTileRanges         render.cu:3510, launch :6812-6824
//   renderCUDA<16,16,2,4>     render.cu:2176, launch :4365-4385 (also <32,16,4,4>,
//                             <32,32,4,8> and the unroll2 form, render.cu:6917-6957)
//   renderCUDAWarpSplit<16|24,16,..,2>  render.cu:4115, launch :4386-4409
//   renderCUDA32x16Split      render.cu:3859, launch :6927-6946
//   renderCUDA_preranges_smem_persistent_lite<16,16,2,4>       render.cu:1717, launch :6537-6573
//   renderCUDA_preranges_smem_persistent_lite_fused<16,16,2,4> render.cu:2026, launch :6616-6652
// The reference's sort.cu does not compile against CUDA 13's CCCL (its
// pre-bound SM90 dispatch type is gone), so ref_sort() below issues the same
// library call that sort.cu:107-125 makes -- cub::DeviceRadixSort::SortPairs
// on (u64 key, u32 value) over bits [0, 32 + msb(tiles)) -- through CUB's
// public entry point.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

namespace {

CUmodule g_pre = nullptr;
CUmodule g_ren = nullptr;
CUdeviceptr g_tile_counter = 0;  // the persistent kernels' module-global queue counter
std::string g_dir;
int* g_pinned = nullptr;         // fetch_num_rendered_async's pinned slot (sort.cu:31-69)
cudaEvent_t g_evt = nullptr;

CUresult load(const std::string& file, CUmodule* m) { return cuModuleLoad(m, (g_dir + "/" + file).c_str()); }

// Find a kernel whose mangled name contains `needle`; optionally return its name.
CUfunction find(CUmodule m, const char* needle, const char** name_out = nullptr)
{
    unsigned n = 0;
    if (cuModuleGetFunctionCount(&n, m) != CUDA_SUCCESS || n == 0) return nullptr;
    CUfunction* fs = new CUfunction[n];
    CUfunction hit = nullptr;
    if (cuModuleEnumerateFunctions(fs, n, m) == CUDA_SUCCESS) {
        for (unsigned i = 0; i < n && !hit; i++) {
            const char* name = nullptr;
            if (cuFuncGetName(&name, fs[i]) == CUDA_SUCCESS && name && strstr(name, needle)) {
                hit = fs[i];
                if (name_out) *name_out = name;
            }
        }
    }
    delete[] fs;
    return hit;
}

// g_tile_counter lives in the same anonymous namespace as the render kernels
// (render.cu:1537); its mangled name is "_ZN9polysplat" + <that namespace's
// length-prefixed name> + "14g_tile_counterE".
void locate_tile_counter()
{
    const char* kname = nullptr;
    if (!find(g_ren, "41renderCUDA_preranges_smem_persistent_liteILi16", &kname) || !kname) return;
    const char* prefix = "_ZN9polysplat";
    if (strncmp(kname, prefix, strlen(prefix)) != 0) return;
    const char* p = kname + strlen(prefix);
    char* end = nullptr;
    long len = strtol(p, &end, 10);
    if (len <= 0 || !end) return;
    std::string var = std::string(prefix) + std::string(p, (end - p) + len) + "14g_tile_counterE";
    size_t bytes = 0;
    if (cuModuleGetGlobal(&g_tile_counter, &bytes, g_ren, var.c_str()) != CUDA_SUCCESS || bytes != 4)
        g_tile_counter = 0;
}

int sm_count()
{
    CUdevice d;
    int n = 0;
    if (cuCtxGetDevice(&d) != CUDA_SUCCESS) return 1;
    cuDeviceGetAttribute(&n, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, d);
    return n > 0 ? n : 1;
}

struct LoadInfo {  // render.cu:396-402, the by-value argument of renderCUDA
    const void* data[32];
    const void* topk_data[32];
    int lg2_scale[32];
};

LoadInfo make_load_info(const void* vals, const float* xy, const float* rgbd, const float* con)
{
    // lane -> source table of render.cu:404-488
    LoadInfo L;
    memset(&L, 0, sizeof L);
    auto set = [&](int lane, const void* p, int s) {
        L.data[lane] = p;
        L.lg2_scale[lane] = s;
    };
    set(0, vals, 2);
    set(4, vals, 2);
    set(8, xy, 3);
    set(9, xy + 1, 3);
    set(12, xy, 3);
    set(13, xy + 1, 3);
    for (int k = 0; k < 3; k++) {
        set(16 + k, rgbd + k, 4);
        set(20 + k, rgbd + k, 4);
    }
    for (int k = 0; k < 4; k++) {
        set(24 + k, con + k, 4);
        set(28 + k, con + k, 4);
    }
    return L;
}

}  // namespace

extern "C" {

// Returns 0 when the reference cubins are loaded.
int ref_open(const char* dir)
{
    if (cuInit(0) != CUDA_SUCCESS) return 1;
    CUcontext ctx = nullptr;
    if (cuCtxGetCurrent(&ctx) != CUDA_SUCCESS || !ctx) return 2;
    g_dir = dir;
    if (!g_pre && load("preprocess.cubin", &g_pre) != CUDA_SUCCESS) return 3;
    if (!g_ren && load("render.cubin", &g_ren) != CUDA_SUCCESS) return 5;
    if (!g_pinned) {
        if (cudaHostAlloc((void**)&g_pinned, sizeof(int), cudaHostAllocDefault) != cudaSuccess) return 6;
        cudaEventCreateWithFlags(&g_evt, cudaEventDisableTiming);
    }
    locate_tile_counter();
    return find(g_pre, "14preprocessCUDAE") ? 0 : 4;
}

// 1 when the persistent kernels' counter was found (no module reload per launch).
int ref_has_tile_counter(void) { return g_tile_counter != 0; }

int ref_preprocess(int P, const void* pos, const void* opacity, const void* shs, int shs_half, const float* view16,
                   const float* proj16, const float* campos3, int W, int H, int bx, int by, float tanx, float tany,
                   float fx, float fy, void* xy, void* cov3d, void* rgbd, void* con, void* counter, void* keys,
                   void* vals, void* stream)
{
    CUfunction f = find(g_pre, "14preprocessCUDAE");
    if (!f) return 10;
    if (P <= 0) return 0;
    unsigned char half = shs_half ? 1 : 0;
    float view[16], proj[16], cam[3];
    memcpy(view, view16, sizeof view);
    memcpy(proj, proj16, sizeof proj);
    memcpy(cam, campos3, sizeof cam);
    unsigned grid[3] = {(unsigned)((W + bx - 1) / bx), (unsigned)((H + by - 1) / by), 1u};
    void* packed = nullptr;
    void* args[] = {&P,   (void*)&pos, (void*)&opacity, (void*)&shs, &half, view,   proj, cam,  &W,
                    &H,   &bx,         &by,             &tanx,       &tany, &fx,    &fy,  &xy,  &cov3d,
                    &rgbd, &con,       &packed,         &counter,    &keys, &vals,  grid};
    CUresult r = cuLaunchKernel(f, (P + 127) / 128, 1, 1, 8, 4, 4, 0, (CUstream)stream, args, nullptr);
    return r == CUDA_SUCCESS ? 0 : 20 + (int)r;
}

int ref_tile_ranges(int M, const void* keys, int tiles, void* ranges, void* stream)
{
    CUfunction f = find(g_ren, "17computeTileRangesE");
    if (!f) return 31;
    void* args[] = {(void*)&keys, &M, &tiles, &ranges};
    CUresult r = cuLaunchKernel(f, (tiles + 255) / 256, 1, 1, 256, 1, 1, 0, (CUstream)stream, args, nullptr);
    return r == CUDA_SUCCESS ? 0 : 40 + (int)r;
}

// which: 0 = persistent lite (ranges), 1 = persistent lite fused (keys), 2 = default renderCUDA (keys),
// 3-8 = the other one-block-per-tile renders (keys; see the table below)
int ref_render(int which, int M, int W, int H, const void* xy, const void* rgbd, const void* con, const void* keys,
               const void* vals, const void* ranges, const float* bg3, void* out, void* stream)
{
    CUmodule m = g_ren;
    bool fresh = false;
    if ((which == 0 || which == 1) && !g_tile_counter) {
        // counter not found: a fresh module starts it at zero
        if (load("render.cubin", &m) != CUDA_SUCCESS) return 50;
        fresh = true;
    }
    const int x_blocks = (W + 15) / 16, y_blocks = (H + 15) / 16, tiles = x_blocks * y_blocks;
    float bg[3] = {bg3[0], bg3[1], bg3[2]};
    CUresult r = CUDA_ERROR_NOT_FOUND;
    if (which == 0 || which == 1) {
        CUfunction f = which == 0 ? find(m, "41renderCUDA_preranges_smem_persistent_liteILi16ELi16ELi2ELi4E")
                                  : find(m, "47renderCUDA_preranges_smem_persistent_lite_fusedILi16ELi16ELi2ELi4E");
        if (f) {
            // render.cu:6628-6638: occupancy query and counter reset on every call
            int per_sm = 0;
            cuOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, 32, 0);
            int grid = sm_count() * (per_sm > 0 ? per_sm : 1);
            if (grid > tiles) grid = tiles;
            if (!fresh) cuMemsetD32Async(g_tile_counter, 0u, 1, (CUstream)stream);
            if (which == 0) {
                void* args[] = {(void*)&vals, &W, &H, (void*)&x_blocks, (void*)&tiles, (void*)&xy, (void*)&rgbd,
                                (void*)&con,  (void*)&ranges, bg, &out};
                r = cuLaunchKernel(f, grid, 1, 1, 8, 4, 1, 0, (CUstream)stream, args, nullptr);
            } else {
                void* args[] = {(void*)&keys, &M,          (void*)&vals, &W, &H, (void*)&x_blocks, (void*)&tiles,
                                (void*)&xy,   (void*)&rgbd, (void*)&con, bg, &out};
                r = cuLaunchKernel(f, grid, 1, 1, 8, 4, 1, 0, (CUstream)stream, args, nullptr);
            }
        }
    } else if (which >= 2 && which <= 8) {
        // one block per tile, ranges searched in the keys (render.cu:4365-4409, 6897-6946)
        struct Shape {
            const char* needle;
            int bx, by, tx, ty;
        };
        static const Shape shapes[] = {
            {"10renderCUDAILi16ELi16ELi2ELi4ELb0ELb0E", 16, 16, 8, 4},         // 2: render_16x16
            {"10renderCUDAILi32ELi16ELi4ELi4ELb0ELb0E", 32, 16, 8, 4},         // 3: render_32x16
            {"10renderCUDAILi32ELi32ELi4ELi8ELb0ELb0E", 32, 32, 8, 4},         // 4: render_32x32
            {"10renderCUDAILi16ELi16ELi2ELi4ELb1ELb0E", 16, 16, 8, 4},         // 5: render_16x16_unroll2
            {"19renderCUDAWarpSplitILi16ELi16ELi2ELi2ELi2E", 16, 16, 8, 8},    // 6: render_16x16_split
            {"19renderCUDAWarpSplitILi24ELi16ELi3ELi2ELi2E", 24, 16, 8, 8},    // 7: render_24x16_split
            {"20renderCUDA32x16Split", 32, 16, 16, 4},                          // 8: render_32x16_split
        };
        const Shape& sh = shapes[which - 2];
        CUfunction f = find(m, sh.needle);
        if (f) {
            const int gx = (W + sh.bx - 1) / sh.bx, gy = (H + sh.by - 1) / sh.by;
            LoadInfo info = make_load_info(vals, (const float*)xy, (const float*)rgbd, (const float*)con);
            void* args[] = {(void*)&keys, &M, (void*)&vals, &W, &H, (void*)&gx, (void*)&xy, (void*)&rgbd,
                            (void*)&con,  &info, bg, &out};
            r = cuLaunchKernel(f, gx, gy, 1, sh.tx, sh.ty, 1, 0, (CUstream)stream, args, nullptr);
        }
    }
    int rc = r == CUDA_SUCCESS ? 0 : 60 + (int)r;
    if (fresh) {
        cuStreamSynchronize((CUstream)stream);
        cuModuleUnload(m);
    }
    return rc;
}

// Bytes of temporary storage CUB needs for `n` pairs (sort.cu:127-133).
size_t ref_sort_temp_bytes(int n)
{
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs<uint64_t, uint32_t>(nullptr, bytes, nullptr, nullptr, nullptr, nullptr, n, 0, 64);
    return bytes;
}

// sort.cu:107-125: end_bit = 32 + msb(tiles); the count comes from the host.
int ref_sort(int n, int end_bit, void* temp, size_t temp_bytes, const void* keys_in, const void* vals_in,
             void* keys_out, void* vals_out, void* stream)
{
    cudaError_t e = cub::DeviceRadixSort::SortPairs(temp, temp_bytes, (const uint64_t*)keys_in, (uint64_t*)keys_out,
                                                    (const uint32_t*)vals_in, (uint32_t*)vals_out, n, 0, end_bit,
                                                    (cudaStream_t)stream);
    return e == cudaSuccess ? 0 : 70 + (int)e;
}

// ---- the reference's ES ("early sorting") steps (csrc/pybind.cpp:183-330) ----
// Pass A and pass B are the reference's kernels from the cubin, launched as
// its host wrappers do (preprocess.cu:1335-1446: grid (P + 127) / 128, block
// (8, 4, 4)).  The steps between them are the CUB calls of sort.cu:204-285
// issued through CUB's public entry points, with this file's own one-line
// helper kernels for the identity, gather, total and key-rebuild steps.

// preprocess_es_pass_a{,_half_sh} (preprocess.cu:1335-1402)
int ref_es_pass_a(int P, const void* pos, const void* opacity, const void* shs, int shs_half, const float* view16,
                  const float* proj16, const float* campos3, int W, int H, int bx, int by, float tanx, float tany,
                  float fx, float fy, void* xy, void* cov3d, void* rgbd, void* con, void* tiles_per_gauss,
                  void* conic_power_raw, void* depth_natural, void* rect_bounds, void* stream)
{
    CUfunction f = find(g_pre, "23preprocessCUDA_ES_PassAE");
    if (!f) return 11;
    if (P <= 0) return 0;
    unsigned char half = shs_half ? 1 : 0;
    float view[16], proj[16], cam[3];
    memcpy(view, view16, sizeof view);
    memcpy(proj, proj16, sizeof proj);
    memcpy(cam, campos3, sizeof cam);
    unsigned grid[3] = {(unsigned)((W + bx - 1) / bx), (unsigned)((H + by - 1) / by), 1u};
    void* packed = nullptr;
    void* args[] = {&P,    (void*)&pos, (void*)&opacity, (void*)&shs, &half,          view,
                    proj,  cam,         &W,              &H,          &bx,            &by,
                    &tanx, &tany,       &fx,             &fy,         &xy,            &cov3d,
                    &rgbd, &con,        &packed,         &tiles_per_gauss, &conic_power_raw, &depth_natural,
                    &rect_bounds, grid};
    CUresult r = cuLaunchKernel(f, (P + 127) / 128, 1, 1, 8, 4, 4, 0, (CUstream)stream, args, nullptr);
    return r == CUDA_SUCCESS ? 0 : 20 + (int)r;
}

// preprocess_es_pass_b (preprocess.cu:1407-1446)
int ref_es_pass_b(int P, int W, int H, int bx, int by, const void* perm, const void* cum, const void* tpg_sorted,
                  const void* xy, const void* cpr, const void* rb, void* tile_keys, void* vals, void* stream)
{
    CUfunction f = find(g_pre, "23preprocessCUDA_ES_PassBE");
    if (!f) return 12;
    if (P <= 0) return 0;
    unsigned grid[3] = {(unsigned)((W + bx - 1) / bx), (unsigned)((H + by - 1) / by), 1u};
    void* args[] = {&P,          &bx,         &by,        (void*)&perm, (void*)&cum,    (void*)&tpg_sorted,
                    (void*)&xy,  (void*)&cpr, (void*)&rb, &tile_keys,   &vals,          grid};
    CUresult r = cuLaunchKernel(f, (P + 127) / 128, 1, 1, 8, 4, 4, 0, (CUstream)stream, args, nullptr);
    return r == CUDA_SUCCESS ? 0 : 20 + (int)r;
}

}  // extern "C"

namespace {
__global__ void es_identity(int P, uint32_t* id)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P) id[i] = (uint32_t)i;
}
__global__ void es_gather(int P, const uint32_t* perm, const int32_t* src, int32_t* dst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P) dst[i] = src[perm[i]];
}
__global__ void es_total(int P, const int32_t* cum, const int32_t* cnt, int32_t* out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *out = P > 0 ? cum[P - 1] + cnt[P - 1] : 0;
}
__global__ void es_rebuild(int M, const uint32_t* t32, uint64_t* k64)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < M) k64[i] = (uint64_t)t32[i] << 32;
}
unsigned higher_msb(unsigned n)  // getHigherMsb (sort.cu:14-29)
{
    unsigned msb = 16, step = 16;
    while (step > 1) {
        step /= 2;
        if (n >> msb) msb += step;
        else msb -= step;
    }
    if (n >> msb) msb++;
    return msb;
}
}  // namespace

extern "C" {

// Temporary bytes of the three CUB calls (sort.cu:127-149, 186-191).
size_t ref_es_depth_sort_temp_bytes(int P)
{
    size_t b = 0;
    cub::DeviceRadixSort::SortPairs<float, uint32_t>(nullptr, b, nullptr, nullptr, nullptr, nullptr, P, 0, 32);
    return b;
}
size_t ref_es_scan_temp_bytes(int P)
{
    size_t b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b, (int32_t*)nullptr, (int32_t*)nullptr, P);
    return b;
}
size_t ref_es_tile_sort_temp_bytes(int M)
{
    size_t b = 0;
    cub::DeviceRadixSort::SortPairs<uint32_t, uint32_t>(nullptr, b, nullptr, nullptr, nullptr, nullptr, M, 0, 32);
    return b;
}

// es_depth_sort_and_scan (sort.cu:204-245)
int ref_es_depth_sort_and_scan(int P, const void* tiles_per_gauss, const void* depth_natural, void* identity,
                               void* perm, void* depth_sorted, void* tpg_sorted, void* cum, void* total,
                               void* sort_temp, size_t sort_bytes, void* scan_temp, size_t scan_bytes, void* stream)
{
    if (P <= 0) return 0;
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = (P + 255) / 256;
    es_identity<<<nb, 256, 0, s>>>(P, (uint32_t*)identity);
    size_t b = sort_bytes;
    cudaError_t e = cub::DeviceRadixSort::SortPairs<float, uint32_t>(
        sort_temp, b, (const float*)depth_natural, (float*)depth_sorted, (const uint32_t*)identity, (uint32_t*)perm, P,
        0, 32, s);
    if (e != cudaSuccess) return 80 + (int)e;
    es_gather<<<nb, 256, 0, s>>>(P, (const uint32_t*)perm, (const int32_t*)tiles_per_gauss, (int32_t*)tpg_sorted);
    b = scan_bytes;
    e = cub::DeviceScan::ExclusiveSum(scan_temp, b, (const int32_t*)tpg_sorted, (int32_t*)cum, P, s);
    if (e != cudaSuccess) return 90 + (int)e;
    es_total<<<1, 32, 0, s>>>(P, (const int32_t*)cum, (const int32_t*)tpg_sorted, (int32_t*)total);
    return cudaGetLastError() == cudaSuccess ? 0 : 99;
}

// es_tile_sort (sort.cu:248-285)
int ref_es_tile_sort(int M, int W, int H, int bx, int by, const void* tk_u, const void* v_u, void* tk_s, void* v_s,
                     void* keys64, void* temp, size_t temp_bytes, void* stream)
{
    if (M <= 0) return 0;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned tiles = (unsigned)(((W + bx - 1) / bx) * ((H + by - 1) / by));
    size_t b = temp_bytes;
    cudaError_t e = cub::DeviceRadixSort::SortPairs<uint32_t, uint32_t>(
        temp, b, (const uint32_t*)tk_u, (uint32_t*)tk_s, (const uint32_t*)v_u, (uint32_t*)v_s, M, 0,
        (int)higher_msb(tiles), s);
    if (e != cudaSuccess) return 80 + (int)e;
    es_rebuild<<<(M + 255) / 256, 256, 0, s>>>(M, (const uint32_t*)tk_s, (uint64_t*)keys64);
    return cudaGetLastError() == cudaSuccess ? 0 : 99;
}

// The reference's E2E forward (csrc/pybind.cpp:1085-1149): memset counter,
// preprocess (FP16 SH), pinned read-back of the key count, CUB sort, persistent
// fused render.  Returns the key count, or a negative code.
int ref_forward_e2e(int P, const void* pos, const void* shs_half, const void* opacity, void* cov3d, const float* view16,
                    const float* proj16, const float* campos3, int W, int H, float fx, float fy, void* counter,
                    void* sort_temp, size_t sort_temp_bytes, void* ku, void* vu, void* ks, void* vs, void* xy,
                    void* rgbd, void* con, const float* bg3, void* out, void* stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemsetAsync(counter, 0, sizeof(int), s);
    int rc = ref_preprocess(P, pos, opacity, shs_half, 1, view16, proj16, campos3, W, H, 16, 16, W / (2.0f * fx),
                            H / (2.0f * fy), fx, fy, xy, cov3d, rgbd, con, counter, ku, vu, stream);
    if (rc) return -rc;
    cudaMemcpyAsync(g_pinned, counter, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaEventRecord(g_evt, s);
    cudaEventSynchronize(g_evt);
    const int num = *g_pinned;
    const int tiles = ((W + 15) / 16) * ((H + 15) / 16);
    int msb = 16, step = 16;  // getHigherMsb, sort.cu:14-29
    while (step > 1) {
        step /= 2;
        if ((unsigned)tiles >> msb) msb += step;
        else msb -= step;
    }
    if ((unsigned)tiles >> msb) msb++;
    rc = ref_sort(num, 32 + msb, sort_temp, sort_temp_bytes, ku, vu, ks, vs, stream);
    if (rc) return -rc;
    rc = ref_render(1, num, W, H, xy, rgbd, con, ks, vs, nullptr, bg3, out, stream);
    if (rc) return -rc;
    return num;
}

}  // extern "C"
