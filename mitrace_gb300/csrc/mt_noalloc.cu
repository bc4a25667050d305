// mt_noalloc.cu - a render entry point that allocates nothing.
//
// Some callers cannot allocate GPU memory when they need a render: a host
// application with a fixed GPU memory budget that was reserved up front, a
// frame loop or host callback that must not block on the allocator (cudaMalloc
// can synchronise the device), or a process whose allocator is hooked by
// another library that forbids allocations during its work.  For them,
// mt_render_rows_noalloc renders a band of image rows with exactly the kernels
// mt_render_device uses, but every scratch buffer of the wavefront (path state,
// path queues, shadow-ray queue, per-sample planes, counters) lives in one
// file-scope device array of fixed size, g_noalloc_scratch below.  The scene
// itself was uploaded by mt_create beforehand; the caller passes the output.
//
// Limits and rules:
//   * one call renders at most MT_NOALLOC_MAX_PATHS paths: (row1 - row0) *
//     width * samples must not exceed it (larger requests return MT_ERR_INVALID);
//   * the array (MT_NOALLOC_SCRATCH_BYTES, about 16 MiB) exists on every GPU
//     that loads this library, for as long as the process lives;
//   * every call shares that one array, which keeps the previous call's
//     contents; the counters that must start at zero are cleared on the stream
//     at the start of each call.  Calls whose work overlaps on the GPU (two
//     streams, two host threads, two handles) race on the array: serialise them;
//   * mt_get_stats counts the samples of these calls but not their rays;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, that device current).  Make that
//     first call before any stream capture begins.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/mitrace_gpu.h"
#include "mt_device.cuh"
#include "mt_internal.h"
#include "mt_kernels.h"

namespace {

constexpr uint64_t kMaxPaths = MT_NOALLOC_MAX_PATHS;
// Layout (bytes): 11 float4 path planes, 3 float4 shadow planes, 2 u32 queues,
// 3 float sample planes, then 8 u32 counters and 2 u64 ray counters.
constexpr uint64_t kPathBytes = (11 + 3) * 16 + 2 * 4 + 3 * 4;
constexpr uint64_t kCounterOffset = kMaxPaths * kPathBytes;
constexpr uint64_t kScratchBytes = kCounterOffset + 8 * 4 + 2 * 8;
static_assert(kScratchBytes <= MT_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the declared size");

// Device address space only: in host code this name is a host-side shadow,
// never a device address.
static __device__ __align__(256) unsigned char g_noalloc_scratch[MT_NOALLOC_SCRATCH_BYTES];

std::mutex g_mu;
constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {};

// Looks up the device address of g_noalloc_scratch on the current device, once.
cudaError_t scratch_address(void** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" mt_status mt_render_rows_noalloc(mt_handle* h, uint32_t row0, uint32_t row1, float* d_rgb_out,
                                            void* cuda_stream)
{
    using namespace mt;
    const DevScene* S = internal_scene(h);
    if (!S || !d_rgb_out) return internal_error(MT_ERR_INVALID, "null handle or output");
    if (internal_busy(h)) return internal_error(MT_ERR_STATE, "an asynchronous render is running");
    if (row0 >= row1 || row1 > S->height)
        return internal_error(MT_ERR_INVALID, "rows must satisfy row0 < row1 <= height");
    if (S->debug_mode) return internal_error(MT_ERR_INVALID, "debug render modes need mt_render_device");
    const uint64_t band_pix = static_cast<uint64_t>(row1 - row0) * S->width;
    const uint64_t paths = band_pix * S->spp;
    if (paths > kMaxPaths)
        return internal_error(MT_ERR_INVALID,
                              "rows x width x samples = " + std::to_string(paths) +
                                  " exceeds the allocation-free limit of " + std::to_string(kMaxPaths) +
                                  " paths per call (MT_NOALLOC_MAX_PATHS)");
    void* base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess)
        return internal_error(MT_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);

    const uint64_t P = kMaxPaths;
    float4* f4 = static_cast<float4*>(base);
    PathState ps;
    ps.ro = f4 + 0 * P;
    ps.rd = f4 + 1 * P;
    ps.cur = f4 + 2 * P;
    ps.tot = f4 + 3 * P;
    ps.prev = f4 + 4 * P;
    ps.emit = f4 + 5 * P;
    ps.direct = f4 + 6 * P;
    ps.indirect = f4 + 7 * P;
    ps.sky = f4 + 8 * P;
    ps.hitA = f4 + 9 * P;
    ps.hitB = reinterpret_cast<uint4*>(f4 + 10 * P);
    ShadowQueue sq;
    sq.o = f4 + 11 * P;
    sq.d = f4 + 12 * P;
    sq.c = f4 + 13 * P;
    uint32_t* q = reinterpret_cast<uint32_t*>(f4 + 14 * P);
    float* planes = reinterpret_cast<float*>(q + 2 * P);
    unsigned char* tail = static_cast<unsigned char*>(base) + kCounterOffset;
    WaveBuffers w;
    w.q[0] = q;
    w.q[1] = q + P;
    w.counts = reinterpret_cast<uint32_t*>(tail);
    w.rays = reinterpret_cast<unsigned long long*>(tail + 8 * 4);
    w.sr = planes;
    w.sg = planes + P;
    w.sb = planes + 2 * P;

    // counters left over from the previous call start at zero
    e = cudaMemsetAsync(tail, 0, 8 * 4 + 2 * 8, st);
    if (e == cudaSuccess)
        e = launch_batch(*S, ps, sq, w, 0, static_cast<uint32_t>(paths), static_cast<uint32_t>(band_pix),
                         row0 * S->width, st, nullptr, nullptr);
    if (e == cudaSuccess)
        e = launch_resolve(*S, w, static_cast<uint32_t>(band_pix), row0 * S->width, d_rgb_out, st, nullptr);
    if (e != cudaSuccess) return internal_error(MT_ERR_CUDA, cudaGetErrorString(e));
    // mt_get_stats counts the call's camera samples; its ray counters stay in
    // the shared scratch array (reading them back would need a host copy that
    // waits for the GPU), so the rays of allocation-free calls are not counted
    internal_count_samples(h, paths);
    return MT_OK;
}
